// K1: the stochastic-Galerkin operator apply on sm_103a.
//
// Computes, for every device row i (mul!(Ax, S, x), src/modelproblems/
// solvers_poisson_primal.jl:86-124):
//     Y[i, mu] = sum_j K_0[i,j] X[j, mu] + sum_{m, nu} G[(m-1)P+mu, nu] sum_j K_m[i,j] X[j, nu]
// and Y[i, :] = 0 on Dirichlet rows.  The reference performs one full SpMV per
// nonzero of G (solvers_poisson_primal.jl:108-115); here every CSR nonzero of
// the shared pattern is read once and applied to all modes:
//   phase 1 (per nonzero, per pair q = (m, nu) of the pair list Q):
//       acc[q] += K_m[i, j] * X[j, nu]
//   phase 2 (per output mode mu):
//       Y[i, mu] = acc[(0, mu)] + sum_{(g, q) in comb(mu)} g * acc[q]
// Pairs (m, nu) exist only where column nu of G_m is nonzero, so the flop
// count is 2 nnz (P + sum_m nzcols(G_m)) + 2 n nnz(G), the minimum for an
// assembled operator.
//
// Mapping: one warp per row, pairs spread over the lanes (lane-strided), the
// gathered mode vector X[j, :] and the M+1 values of the nonzero staged in the
// warp's shared memory, the per-row pair accumulators stored to shared memory
// for phase 2.  Per-block FP64 partials of X .* Y (the p'Ap of CG) are fused
// into the epilogue.
#include <algorithm>
#include <cstring>

#include "sgfem_internal.h"

namespace {

constexpr int WPB = 4;  // warps per block

template <typename T> struct Vec16;
template <> struct Vec16<float> { using type = float4; static constexpr int n = 4; };
template <> struct Vec16<double> { using type = double2; static constexpr int n = 2; };

template <typename T, int QT>
__global__ void __launch_bounds__(WPB * 32)
k_apply(const int* __restrict__ rowptr, const int* __restrict__ col, const T* __restrict__ vals, int M1,
        const T* __restrict__ X, T* __restrict__ Y, int n, int P, int ld, const unsigned char* __restrict__ bmask,
        const int* __restrict__ qtab, int Qn, const int* __restrict__ combptr, const int* __restrict__ combq,
        const T* __restrict__ combg, double* __restrict__ partials, const KrylovScalars* __restrict__ scal) {
    if (scal && scal->done) return;
    extern __shared__ unsigned char smem_raw[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int per_warp = (ld + (M1 + 1) + Qn + 3) & ~3;  // elements of T, 16-byte multiple per slice
    T* su = reinterpret_cast<T*>(smem_raw) + (size_t)warp * per_warp;
    T* sc = su + ld;
    T* sacc = sc + M1 + 1;
    __shared__ double red[WPB];

    if (lane == 0) sc[M1] = T(0);  // zero slot for padded pairs
    using V = typename Vec16<T>::type;
    const int nvec = ld / Vec16<T>::n;
    double dot = 0.0;

    for (int row = blockIdx.x * WPB + warp; row < n; row += gridDim.x * WPB) {
        T* yrow = Y + (size_t)row * ld;
        if (bmask[row]) {
            for (int c = lane; c < ld; c += 32) yrow[c] = T(0);
            continue;
        }
        const int nz0 = rowptr[row], nz1 = rowptr[row + 1];
        for (int base = 0; base < Qn; base += QT * 32) {
            int om[QT], on[QT];
#pragma unroll
            for (int t = 0; t < QT; ++t) {
                const int q = base + t * 32 + lane;
                if (q < Qn) {
                    const int e = qtab[q];
                    om[t] = e >> 16;
                    on[t] = e & 0xffff;
                } else {
                    om[t] = M1;
                    on[t] = 0;
                }
            }
            T acc[QT];
#pragma unroll
            for (int t = 0; t < QT; ++t) acc[t] = T(0);
            for (int nz = nz0; nz < nz1; ++nz) {
                const int j = col[nz];
                const V* xs = reinterpret_cast<const V*>(X + (size_t)j * ld);
                V* sv = reinterpret_cast<V*>(su);
                for (int c = lane; c < nvec; c += 32) sv[c] = __ldg(xs + c);
                for (int m = lane; m < M1; m += 32) sc[m] = vals[(size_t)nz * M1 + m];
                __syncwarp();
#pragma unroll
                for (int t = 0; t < QT; ++t) acc[t] = fma(sc[om[t]], su[on[t]], acc[t]);
                __syncwarp();
            }
#pragma unroll
            for (int t = 0; t < QT; ++t) {
                const int q = base + t * 32 + lane;
                if (q < Qn) sacc[q] = acc[t];
            }
        }
        __syncwarp();
        const T* xrow = X + (size_t)row * ld;
        T rowdot = T(0);  // per-row products in the working precision, rows summed in FP64
        for (int mu = lane; mu < ld; mu += 32) {
            T y = T(0);
            if (mu < P) {
                y = sacc[mu];
                for (int e = combptr[mu]; e < combptr[mu + 1]; ++e) y = fma(combg[e], sacc[combq[e]], y);
            }
            yrow[mu] = y;
            if (partials) rowdot = fma(xrow[mu], y, rowdot);
        }
        dot += (double)rowdot;
        __syncwarp();
    }
    if (partials) {
        for (int o = 16; o > 0; o >>= 1) dot += __shfl_down_sync(0xffffffffu, dot, o);
        if (lane == 0) red[warp] = dot;
        __syncthreads();
        if (threadIdx.x == 0) {
            double s = 0.0;
            for (int w = 0; w < WPB; ++w) s += red[w];
            partials[blockIdx.x] = s;
        }
    }
}

template <typename T, int QT>
int launch_qt(sgfem_context* ctx, const T* vals, const T* combg, const void* X, void* Y, double* partials,
              int grid, const KrylovScalars* scal) {
    const size_t per_warp = ((size_t)ctx->ld + ctx->M1 + 1 + ctx->Qn + 3) & ~(size_t)3;
    const size_t smem = per_warp * sizeof(T) * WPB;
    if (grid == 0) {  // configuration call
        if (smem > 48 * 1024)
            SG_CUDA(ctx, cudaFuncSetAttribute(k_apply<T, QT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        return SGFEM_OK;
    }
    k_apply<T, QT><<<grid, WPB * 32, smem, ctx->stream>>>(
        ctx->d_rowptr, ctx->d_col, vals, ctx->M1, (const T*)X, (T*)Y, (int)ctx->n, (int)ctx->P, (int)ctx->ld,
        ctx->d_bmask, ctx->d_qtab, ctx->Qn, ctx->d_combptr, ctx->d_combq, combg, partials, scal);
    SG_LAUNCHED(ctx);
    return SGFEM_OK;
}

template <typename T>
int launch_t(sgfem_context* ctx, const T* vals, const T* combg, const void* X, void* Y, double* partials, int grid,
             const KrylovScalars* scal) {
    const int need = (ctx->Qn + 31) / 32;
    if (need <= 1) return launch_qt<T, 1>(ctx, vals, combg, X, Y, partials, grid, scal);
    if (need <= 2) return launch_qt<T, 2>(ctx, vals, combg, X, Y, partials, grid, scal);
    if (need <= 4) return launch_qt<T, 4>(ctx, vals, combg, X, Y, partials, grid, scal);
    if (need <= 8) return launch_qt<T, 8>(ctx, vals, combg, X, Y, partials, grid, scal);
    if (need <= 12) return launch_qt<T, 12>(ctx, vals, combg, X, Y, partials, grid, scal);
    if (need <= 16) return launch_qt<T, 16>(ctx, vals, combg, X, Y, partials, grid, scal);
    if (need <= 20) return launch_qt<T, 20>(ctx, vals, combg, X, Y, partials, grid, scal);
    return launch_qt<T, 24>(ctx, vals, combg, X, Y, partials, grid, scal);  // rounds for larger Q
}

}  // namespace

int sg_apply_configure(sgfem_context* ctx) {
    SG_TRY(launch_t<double>(ctx, ctx->d_val64, ctx->d_combg64, nullptr, nullptr, nullptr, 0, nullptr));
    SG_TRY(launch_t<float>(ctx, ctx->d_val32, ctx->d_combg32, nullptr, nullptr, nullptr, 0, nullptr));
    return SGFEM_OK;
}

int sg_launch_apply_samples(sgfem_context* ctx, int precision, const void* X, void* Y, double* dot_partials,
                            int* nblocks, const KrylovScalars* skip_if_done);

int sg_launch_apply(sgfem_context* ctx, int precision, const void* X, void* Y, double* dot_partials, int* nblocks,
                    const KrylovScalars* skip_if_done) {
    if (ctx->batched) return sg_launch_apply_samples(ctx, precision, X, Y, dot_partials, nblocks, skip_if_done);
    const size_t per_warp = ((size_t)ctx->ld + ctx->M1 + 1 + ctx->Qn + 3) & ~(size_t)3;
    const size_t smem = per_warp * sg_elem_bytes(precision) * WPB;
    if (smem > 200 * 1024)
        return sg_fail(ctx, SGFEM_ERR_UNSUPPORTED, "apply: per-row pair list too large for shared memory");
    if (precision == SGFEM_FP32 && sg_jit_accepts(ctx, X)) {
        const int jgrid = sg_jit_grid(ctx);
        if (nblocks) *nblocks = jgrid;
        return sg_jit_launch(ctx, X, Y, dot_partials, jgrid, skip_if_done);
    }
    int grid = (int)std::min<int64_t>((ctx->n + WPB - 1) / WPB, (int64_t)ctx->num_sms * 8);
    if (grid < 1) grid = 1;
    if (nblocks) *nblocks = grid;
    if (precision == SGFEM_FP64)
        return launch_t<double>(ctx, ctx->d_val64, ctx->d_combg64, X, Y, dot_partials, grid, skip_if_done);
    return launch_t<float>(ctx, ctx->d_val32, ctx->d_combg32, X, Y, dot_partials, grid, skip_if_done);
}

// ---------------------------------------------------------------------------
// Block-diagonal sample operator (sgfem_set_samples): column s of Y is
//   Y[i, s] = sum_j (K_0[i,j] + sum_{m<=M} y_{s,m} K_m[i,j]) X[j, s],
// Dirichlet rows zero.  Warp per (row, 32-sample chunk), lane = sample; the
// lane's coefficients y_{s,0..M} live in registers (MMAX >= M+1), the M+1
// values of a nonzero are read with a warp-uniform address.  This is the
// operator of the S deterministic problems of the sampling error
// (src/sampling_error.jl:118-128, src/modelproblems/poisson_primal.jl:14-35).
namespace {

template <typename T, int MMAX>
__global__ void __launch_bounds__(128)
k_apply_samples(const int* __restrict__ rowptr, const int* __restrict__ col, const T* __restrict__ vals, int M1,
                const T* __restrict__ ycoef, const T* __restrict__ X, T* __restrict__ Y, int n, int S, int ld,
                const unsigned char* __restrict__ bmask, double* __restrict__ partials,
                const KrylovScalars* __restrict__ scal) {
    if (scal && scal->done) return;
    __shared__ double red[4];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int nchunk = (ld + 31) / 32;
    const long long items = (long long)n * nchunk;
    double dot = 0.0;
    for (long long it = (long long)blockIdx.x * 4 + warp; it < items; it += (long long)gridDim.x * 4) {
        const int row = (int)(it / nchunk), ch = (int)(it - (long long)row * nchunk);
        const int s = ch * 32 + lane;
        T y[MMAX];
#pragma unroll
        for (int m = 0; m < MMAX; ++m) y[m] = (s < S && m < M1) ? ycoef[(size_t)s * M1 + m] : T(0);
        T acc = T(0);
        if (!bmask[row]) {
            for (int nz = rowptr[row]; nz < rowptr[row + 1]; ++nz) {
                const int j = col[nz];
                const T* v = vals + (size_t)nz * M1;
                T c = T(0);
#pragma unroll
                for (int m = 0; m < MMAX; ++m)
                    if (m < M1) c = fma(y[m], v[m], c);
                if (s < ld) acc = fma(c, X[(size_t)j * ld + s], acc);
            }
        }
        if (s < ld) {
            Y[(size_t)row * ld + s] = acc;
            if (partials) dot += (double)X[(size_t)row * ld + s] * (double)acc;
        }
    }
    if (partials) {
        for (int o = 16; o > 0; o >>= 1) dot += __shfl_down_sync(0xffffffffu, dot, o);
        if (lane == 0) red[warp] = dot;
        __syncthreads();
        if (threadIdx.x == 0) partials[blockIdx.x] = red[0] + red[1] + red[2] + red[3];
    }
}

// the same with K(y_s) precomputed ([nz][ld]): per nonzero one coefficient load
// (contiguous over the warp's samples) and one FMA
template <typename T>
__global__ void __launch_bounds__(128)
k_apply_samples_pre(const int* __restrict__ rowptr, const int* __restrict__ col, const T* __restrict__ kval,
                    const T* __restrict__ X, T* __restrict__ Y, int n, int ld, const unsigned char* __restrict__ bmask,
                    double* __restrict__ partials, const KrylovScalars* __restrict__ scal) {
    if (scal && scal->done) return;
    __shared__ double red[4];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int nchunk = (ld + 31) / 32;
    const long long items = (long long)n * nchunk;
    double dot = 0.0;
    for (long long it = (long long)blockIdx.x * 4 + warp; it < items; it += (long long)gridDim.x * 4) {
        const int row = (int)(it / nchunk), ch = (int)(it - (long long)row * nchunk);
        const int s = ch * 32 + lane;
        if (s >= ld) continue;
        T acc = T(0);
        if (!bmask[row])
            for (int nz = rowptr[row]; nz < rowptr[row + 1]; ++nz)
                acc = fma(kval[(size_t)nz * ld + s], X[(size_t)col[nz] * ld + s], acc);
        Y[(size_t)row * ld + s] = acc;
        if (partials) dot += (double)X[(size_t)row * ld + s] * (double)acc;
    }
    if (partials) {
        for (int o = 16; o > 0; o >>= 1) dot += __shfl_down_sync(0xffffffffu, dot, o);
        if (lane == 0) red[warp] = dot;
        __syncthreads();
        if (threadIdx.x == 0) partials[blockIdx.x] = red[0] + red[1] + red[2] + red[3];
    }
}

// the same with V consecutive samples per lane (16-byte loads: float4 / double2; ld is
// a multiple of 4): four times the bytes in flight per load instruction.  Per sample
// the nonzeros are summed in the same order as above.
template <typename T, int V> struct SampleVec;
template <> struct SampleVec<float, 4> { using type = float4; };
template <> struct SampleVec<double, 2> { using type = double2; };

template <typename T, int V>
__global__ void __launch_bounds__(128)
k_apply_samples_pre_v(const int* __restrict__ rowptr, const int* __restrict__ col, const T* __restrict__ kval,
                      const T* __restrict__ X, T* __restrict__ Y, int n, int ld, const unsigned char* __restrict__ bmask,
                      double* __restrict__ partials, const KrylovScalars* __restrict__ scal) {
    using VT = typename SampleVec<T, V>::type;
    if (scal && scal->done) return;
    __shared__ double red[4];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int nchunk = (ld + 32 * V - 1) / (32 * V);
    const long long items = (long long)n * nchunk;
    double dot = 0.0;
    for (long long it = (long long)blockIdx.x * 4 + warp; it < items; it += (long long)gridDim.x * 4) {
        const int row = (int)(it / nchunk), ch = (int)(it - (long long)row * nchunk);
        const int s = (ch * 32 + lane) * V;
        if (s >= ld) continue;
        T acc[V];
#pragma unroll
        for (int c = 0; c < V; ++c) acc[c] = T(0);
        if (!bmask[row]) {
            const int nz1 = rowptr[row + 1];
            for (int nz = rowptr[row]; nz < nz1; ++nz) {
                T k[V], x[V];
                *reinterpret_cast<VT*>(k) = *reinterpret_cast<const VT*>(kval + (size_t)nz * ld + s);
                *reinterpret_cast<VT*>(x) = *reinterpret_cast<const VT*>(X + (size_t)col[nz] * ld + s);
#pragma unroll
                for (int c = 0; c < V; ++c) acc[c] = fma(k[c], x[c], acc[c]);
            }
        }
        *reinterpret_cast<VT*>(Y + (size_t)row * ld + s) = *reinterpret_cast<const VT*>(acc);
        if (partials) {
            T xr[V];
            *reinterpret_cast<VT*>(xr) = *reinterpret_cast<const VT*>(X + (size_t)row * ld + s);
#pragma unroll
            for (int c = 0; c < V; ++c) dot += (double)xr[c] * (double)acc[c];
        }
    }
    if (partials) {
        for (int o = 16; o > 0; o >>= 1) dot += __shfl_down_sync(0xffffffffu, dot, o);
        if (lane == 0) red[warp] = dot;
        __syncthreads();
        if (threadIdx.x == 0) partials[blockIdx.x] = red[0] + red[1] + red[2] + red[3];
    }
}

// K(y_s)[nz] = sum_m y_{s,m} K_m[nz] in FP64, in the order the on-the-fly kernel sums
// (so the FP64 apply is unchanged bit for bit); the FP32 copy rounds the FP64 sum
__global__ void k_combine_samples(const double* __restrict__ vals, int M1, const double* __restrict__ y, long long nnz,
                                  int S, int ld, double* __restrict__ k64, float* __restrict__ k32) {
    const long long total = nnz * ld;
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (long long)gridDim.x * blockDim.x) {
        const long long nz = t / ld;
        const int s = (int)(t - nz * ld);
        double c = 0.0;
        if (s < S)
            for (int m = 0; m < M1; ++m) c = fma(y[(size_t)s * M1 + m], vals[(size_t)nz * M1 + m], c);
        k64[t] = c;
        k32[t] = (float)c;
    }
}

// (hi, lo) float pairs of doubles: hi = fl(x), lo = fl(x - hi), ~48 significant bits
__global__ void k_split_hilo(const double* __restrict__ v, float2* __restrict__ o, long long n) {
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
        const double x = v[t];
        const float h = __double2float_rn(x);
        o[t] = make_float2(h, __double2float_rn(x - (double)h));
    }
}

// K(y_s)[nz] in double-FP32 on the FP32 pipe (FP64 FMAs run at 1/64 of the FP32 rate
// here): per term the exact product of the hi parts (p = a b, e = fma(a, b, -p)) plus
// the cross terms, summed by an error-free two-sum into (hi, lo); relative error of the
// sum ~2^-46 of sum_m |y_{s,m} K_m[nz]|.  Terms in m order, so results are reproducible.
__global__ void k_combine_samples_df(const float2* __restrict__ vhl, int M1, const float2* __restrict__ yhl,
                                     long long nnz, int S, int ld, double* __restrict__ k64, float* __restrict__ k32) {
    const long long total = nnz * ld;
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (long long)gridDim.x * blockDim.x) {
        const long long nz = t / ld;
        const int s = (int)(t - nz * ld);
        float sh = 0.0f, sl = 0.0f;
        if (s < S)
            for (int m = 0; m < M1; ++m) {
                const float2 a = vhl[(size_t)nz * M1 + m], b = yhl[(size_t)s * M1 + m];
                const float p = __fmul_rn(a.x, b.x);
                float e = __fmaf_rn(a.x, b.x, -p);
                e = __fmaf_rn(a.x, b.y, e);
                e = __fmaf_rn(a.y, b.x, e);
                const float u = __fadd_rn(sh, p);
                const float bv = __fsub_rn(u, sh);
                const float err = __fadd_rn(__fsub_rn(sh, __fsub_rn(u, bv)), __fsub_rn(p, bv));
                sl = __fadd_rn(sl, __fadd_rn(err, e));
                sh = u;
            }
        const float h = __fadd_rn(sh, sl);
        const float l = __fsub_rn(sl, __fsub_rn(h, sh));
        k64[t] = (double)h + (double)l;
        k32[t] = h;
    }
}

template <typename T, int MMAX>
int launch_samples_t(sgfem_context* ctx, const T* vals, const T* y, const void* X, void* Y, double* partials,
                     int grid, const KrylovScalars* scal) {
    k_apply_samples<T, MMAX><<<grid, 128, 0, ctx->stream>>>(ctx->d_rowptr, ctx->d_col, vals, ctx->M1, y,
                                                              (const T*)X, (T*)Y, (int)ctx->n, (int)ctx->P,
                                                              (int)ctx->ld, ctx->d_bmask, partials, scal);
    SG_LAUNCHED(ctx);
    return SGFEM_OK;
}

template <typename T>
int launch_samples(sgfem_context* ctx, const T* vals, const T* y, const void* X, void* Y, double* partials, int grid,
                   const KrylovScalars* scal) {
    if (ctx->M1 <= 8) return launch_samples_t<T, 8>(ctx, vals, y, X, Y, partials, grid, scal);
    if (ctx->M1 <= 16) return launch_samples_t<T, 16>(ctx, vals, y, X, Y, partials, grid, scal);
    if (ctx->M1 <= 24) return launch_samples_t<T, 24>(ctx, vals, y, X, Y, partials, grid, scal);
    if (ctx->M1 <= 32) return launch_samples_t<T, 32>(ctx, vals, y, X, Y, partials, grid, scal);
    if (ctx->M1 <= 64) return launch_samples_t<T, 64>(ctx, vals, y, X, Y, partials, grid, scal);
    return sg_fail(ctx, SGFEM_ERR_UNSUPPORTED, "sample operator: more than 63 KLE terms");
}

}  // namespace

int sg_samples_combine(sgfem_context* ctx) {
    if (!ctx->batched || !ctx->d_val64 || !ctx->d_y64) return SGFEM_OK;
    const size_t count = (size_t)ctx->nnz * ctx->ld;
    if (count * (sizeof(double) + sizeof(float)) > ((size_t)4 << 30)) return SGFEM_OK;
    if (!ctx->d_kval64) {
        SG_CUDA(ctx, cudaMalloc((void**)&ctx->d_kval64, std::max<size_t>(count, 1) * sizeof(double)));
        SG_CUDA(ctx, cudaMalloc((void**)&ctx->d_kval32, std::max<size_t>(count, 1) * sizeof(float)));
    }
    const int grid = (int)std::max<int64_t>(1, std::min<int64_t>(((int64_t)count + 255) / 256, (int64_t)ctx->num_sms * 16));
    const char* ecb = getenv("SGFEM_SAMPLES_COMBINE");
    if (ecb && std::strcmp(ecb, "fp64") == 0) {  // exactly rounded FP64 sums on the FP64 pipe
        k_combine_samples<<<grid, 256, 0, ctx->stream>>>(ctx->d_val64, ctx->M1, ctx->d_y64, (long long)ctx->nnz,
                                                         (int)ctx->P, (int)ctx->ld, ctx->d_kval64, ctx->d_kval32);
        SG_LAUNCHED(ctx);
        return SGFEM_OK;
    }
    const long long nv = (long long)ctx->nnz * ctx->M1, ny = (long long)ctx->P * ctx->M1;
    SG_TRY(sg_ensure(ctx, ctx->w_valhl, (size_t)std::max<long long>(nv, 1) * sizeof(float2)));
    SG_TRY(sg_ensure(ctx, ctx->w_yhl, (size_t)std::max<long long>(ny, 1) * sizeof(float2)));
    const int gs = (int)std::max<long long>(1, std::min<long long>((nv + 255) / 256, (long long)ctx->num_sms * 16));
    k_split_hilo<<<gs, 256, 0, ctx->stream>>>(ctx->d_val64, (float2*)ctx->w_valhl.p, nv);
    SG_LAUNCHED(ctx);
    k_split_hilo<<<(int)std::max<long long>(1, (ny + 255) / 256), 256, 0, ctx->stream>>>(ctx->d_y64,
                                                                                       (float2*)ctx->w_yhl.p, ny);
    SG_LAUNCHED(ctx);
    k_combine_samples_df<<<grid, 256, 0, ctx->stream>>>((const float2*)ctx->w_valhl.p, ctx->M1,
                                                        (const float2*)ctx->w_yhl.p, (long long)ctx->nnz, (int)ctx->P,
                                                        (int)ctx->ld, ctx->d_kval64, ctx->d_kval32);
    SG_LAUNCHED(ctx);
    return SGFEM_OK;
}

int sg_launch_apply_samples(sgfem_context* ctx, int precision, const void* X, void* Y, double* dot_partials,
                            int* nblocks, const KrylovScalars* skip_if_done) {
    const int64_t items = ctx->n * ((ctx->ld + 31) / 32);
    int grid = (int)std::min<int64_t>((items + 3) / 4, (int64_t)ctx->num_sms * 8);
    if (grid < 1) grid = 1;
    if (nblocks) *nblocks = grid;
    const char* evec = getenv("SGFEM_SAMPLES_VEC");
    if (ctx->d_kval64 && ctx->ld % 4 == 0 && !(evec && atoi(evec) == 0)) {
        const int V = precision == SGFEM_FP64 ? 2 : 4;
        const int64_t vitems = ctx->n * ((ctx->ld + 32 * V - 1) / (32 * V));
        grid = (int)std::max<int64_t>(1, std::min<int64_t>((vitems + 3) / 4, (int64_t)ctx->num_sms * 8));
        if (nblocks) *nblocks = grid;
        if (precision == SGFEM_FP64)
            k_apply_samples_pre_v<double, 2><<<grid, 128, 0, ctx->stream>>>(ctx->d_rowptr, ctx->d_col, ctx->d_kval64,
                                                                            (const double*)X, (double*)Y, (int)ctx->n,
                                                                            (int)ctx->ld, ctx->d_bmask, dot_partials,
                                                                            skip_if_done);
        else
            k_apply_samples_pre_v<float, 4><<<grid, 128, 0, ctx->stream>>>(ctx->d_rowptr, ctx->d_col, ctx->d_kval32,
                                                                           (const float*)X, (float*)Y, (int)ctx->n,
                                                                           (int)ctx->ld, ctx->d_bmask, dot_partials,
                                                                           skip_if_done);
        SG_LAUNCHED(ctx);
        return SGFEM_OK;
    }
    if (ctx->d_kval64) {
        if (precision == SGFEM_FP64)
            k_apply_samples_pre<double><<<grid, 128, 0, ctx->stream>>>(ctx->d_rowptr, ctx->d_col, ctx->d_kval64,
                                                                       (const double*)X, (double*)Y, (int)ctx->n,
                                                                       (int)ctx->ld, ctx->d_bmask, dot_partials,
                                                                       skip_if_done);
        else
            k_apply_samples_pre<float><<<grid, 128, 0, ctx->stream>>>(ctx->d_rowptr, ctx->d_col, ctx->d_kval32,
                                                                      (const float*)X, (float*)Y, (int)ctx->n,
                                                                      (int)ctx->ld, ctx->d_bmask, dot_partials,
                                                                      skip_if_done);
        SG_LAUNCHED(ctx);
        return SGFEM_OK;
    }
    if (precision == SGFEM_FP64)
        return launch_samples<double>(ctx, ctx->d_val64, ctx->d_y64, X, Y, dot_partials, grid, skip_if_done);
    return launch_samples<float>(ctx, ctx->d_val32, ctx->d_y32, X, Y, dot_partials, grid, skip_if_done);
}
