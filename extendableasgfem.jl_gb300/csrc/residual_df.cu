// Refinement residual of the mixed solver in double-FP32 arithmetic.
//
// The mixed solver (krylov.cu) needs r = b - A x to about 1e-11 of ||b|| after
// every refinement step (x is the FP64 solution; the residual is the next
// step's right-hand side and the final certificate).  On GB300 FP64 runs at
// 1/64 of the FP32 rate and the FP64 apply (apply.cu, k_apply<double>) is
// FP64-pipe-bound.  This kernel evaluates the same pair-list schedule as
// k_apply with every value held as an unevaluated sum hi + lo of two floats
// (about 48 significant bits) on the FP32 pipe:
//   * x and b are split once per refinement step / solve into (hi, lo) float
//     pairs, the K_m values and the G coefficients once per context;
//   * operator rows with vanishing row sums use the difference form
//     sum_j K_ij (x_j - x_i) (the caller checks the row sums), so the
//     cancellation of K x for smooth x is O(1/h) instead of O(1/h^2);
//   * products are exact (p = a*b, e = fma(a, b, -p)), sums use the
//     error-free two-sum; every operation is an explicit _rn intrinsic so that
//     nothing is contracted or reassociated;
//   * the output is r rounded to FP32 (the next FP32 PCG's right-hand side)
//     plus per-block FP64 partials of its squared norm.
// Same mapping as k_apply: warp per row, pairs (m, nu) lane-strided, the
// differences x_j - x_i of a nonzero and its M+1 values staged in the warp's
// shared memory.
#include <algorithm>

#include "sgfem_internal.h"

namespace {

constexpr int DWPB = 4;  // warps per block
constexpr int DMINB = 4;  // resident blocks per SM the register budget is fitted to

struct DF {
    float h, l;
};

__device__ __forceinline__ DF two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return {s, e};
}

// acc += k * d  (k, d, acc as hi + lo)
__device__ __forceinline__ void df_fma(DF& acc, float2 k, float2 d) {
    const float p = __fmul_rn(k.x, d.x);
    const float pe = __fmaf_rn(k.x, d.x, -p);
    const float pl = __fmaf_rn(k.x, d.y, __fmaf_rn(k.y, d.x, pe));
    const DF s = two_sum(acc.h, p);
    acc.l = __fadd_rn(acc.l, __fadd_rn(s.l, pl));
    acc.h = s.h;
}

// (hi, lo) = (fl32(v), fl32(v - fl32(v))) by integer operations on the bit pattern
// (GB300's FP64 conversions and subtraction run at the FP64 rate): hi keeps the top
// 24 bits of the 53-bit significand rounded to nearest even, lo is the signed
// remainder (< 2^29 units of the last place) times 2^(e - 1075).  Magnitudes
// outside [2^-74, 2^126] (where the scale or hi would leave the normal float
// range) take the FP64 path; zero and subnormal doubles give (0, 0).
__device__ __forceinline__ float2 split_f64(double v) {
    const unsigned long long u = (unsigned long long)__double_as_longlong(v);
    const int e = (int)((u >> 52) & 0x7FF);
    if (e == 0) return make_float2(0.f, 0.f);
    if (e < 949 || e > 1149) {
        const float h = __double2float_rn(v);
        return make_float2(h, __double2float_rn(v - (double)h));
    }
    const unsigned long long mant = (u & 0xFFFFFFFFFFFFFull) | (1ull << 52);
    unsigned int q = (unsigned int)(mant >> 29);
    int rem = (int)(mant & 0x1FFFFFFFull);
    if (rem > (1 << 28) || (rem == (1 << 28) && (q & 1u))) {
        q += 1u;
        rem -= (1 << 29);
    }
    int fe = e - 1023 + 127;
    if (q == (1u << 24)) {
        q >>= 1;
        fe += 1;
    }
    const unsigned int sign = (unsigned int)(u >> 63) << 31;
    const float hi = __uint_as_float(sign | ((unsigned int)fe << 23) | (q & 0x7FFFFFu));
    const float scale = __uint_as_float((unsigned int)(e - 948) << 23);  // 2^(e - 1075)
    const float lo = __fmul_rn(__int2float_rn(rem), scale);
    return make_float2(hi, sign ? -lo : lo);
}

// hi/lo split of FP64 values
__global__ void k_split_pairs(const double* __restrict__ src, float2* __restrict__ dst, size_t count) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += (size_t)gridDim.x * blockDim.x) {
        dst[i] = split_f64(src[i]);
    }
}

// x += d (FP64), then (hi, lo) of the new x into xs (interleaved float2)
__global__ void k_add_split(double* __restrict__ x, const double* __restrict__ d, float2* __restrict__ xs,
                            size_t total, int add) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
        const double v = add ? x[i] + d[i] : x[i];
        if (add) x[i] = v;
        xs[i] = split_f64(v);
    }
}

constexpr int DCOL = 5;  // columns per lane staged from registers (ld <= 160); larger ld loads in place

template <int QT>
__global__ void __launch_bounds__(DWPB * 32, DMINB)
k_residual_df(const int* __restrict__ rowptr, const int* __restrict__ col, const float2* __restrict__ vals, int M1,
              const float2* __restrict__ xs, const float2* __restrict__ bs, float* __restrict__ r32, int n, int P,
              int ld, const unsigned char* __restrict__ bmask, const int* __restrict__ qtab, int Qn,
              const int* __restrict__ combptr, const int* __restrict__ combq, const float2* __restrict__ combg,
              int diff, double* __restrict__ partials) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int per_warp = 2 * ld + (M1 + 1) + Qn;  // float2 slots
    float2* sd = reinterpret_cast<float2*>(smem_raw) + (size_t)warp * per_warp;  // x_j - x_i (ld)
    float2* sx = sd + ld;                                                           // own row x_i (ld)
    float2* sc = sx + ld;                                                           // K_m[i, j] (M1 + 1)
    float2* sacc = sc + M1 + 1;                                                     // pair sums (Qn)
    __shared__ double red[DWPB];
    if (lane == 0) sc[M1] = make_float2(0.f, 0.f);  // zero slot for padded pairs
    float acc_t = 0.f;
    for (int row = blockIdx.x * DWPB + warp; row < n; row += gridDim.x * DWPB) {
        float* rrow = r32 + (size_t)row * ld;
        if (bmask[row]) {
            for (int c = lane; c < ld; c += 32) rrow[c] = 0.f;
            continue;
        }
        const float2* xrow = xs + (size_t)row * ld;
        for (int c = lane; c < ld; c += 32) sx[c] = diff ? xrow[c] : make_float2(0.f, 0.f);
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
            DF acc[QT];
#pragma unroll
            for (int t = 0; t < QT; ++t) acc[t] = {0.f, 0.f};
            // the next nonzero's X row and values are loaded while the current one is used
            const bool reg = ld <= 32 * DCOL;
            float2 xn[DCOL];
            float2 vn = make_float2(0.f, 0.f);
            if (nz0 < nz1) {
                const float2* xj = xs + (size_t)col[nz0] * ld;
#pragma unroll
                for (int u = 0; u < DCOL; ++u) {
                    const int c = lane + 32 * u;
                    xn[u] = (reg && c < ld) ? xj[c] : make_float2(0.f, 0.f);
                }
                if (lane < M1) vn = vals[(size_t)nz0 * M1 + lane];
            }
            for (int nz = nz0; nz < nz1; ++nz) {
                __syncwarp();
                if (reg) {
#pragma unroll
                    for (int u = 0; u < DCOL; ++u) {
                        const int c = lane + 32 * u;
                        if (c < ld) {
                            const float2 a = xn[u], b = sx[c];
                            const DF s = two_sum(a.x, -b.x);
                            sd[c] = make_float2(s.h, __fadd_rn(s.l, __fsub_rn(a.y, b.y)));
                        }
                    }
                } else {
                    const float2* xj = xs + (size_t)col[nz] * ld;
                    for (int c = lane; c < ld; c += 32) {
                        const float2 a = xj[c], b = sx[c];
                        const DF s = two_sum(a.x, -b.x);
                        sd[c] = make_float2(s.h, __fadd_rn(s.l, __fsub_rn(a.y, b.y)));
                    }
                }
                if (lane < M1) sc[lane] = vn;
                __syncwarp();
                if (nz + 1 < nz1) {
                    const float2* xj = xs + (size_t)col[nz + 1] * ld;
#pragma unroll
                    for (int u = 0; u < DCOL; ++u) {
                        const int c = lane + 32 * u;
                        if (reg && c < ld) xn[u] = xj[c];
                    }
                    if (lane < M1) vn = vals[(size_t)(nz + 1) * M1 + lane];
                }
#pragma unroll
                for (int t = 0; t < QT; ++t) df_fma(acc[t], sc[om[t]], sd[on[t]]);
            }
#pragma unroll
            for (int t = 0; t < QT; ++t) {
                const int q = base + t * 32 + lane;
                if (q < Qn) sacc[q] = make_float2(acc[t].h, acc[t].l);
            }
        }
        __syncwarp();
        const float2* brow = bs + (size_t)row * ld;
        for (int mu = lane; mu < ld; mu += 32) {
            float rv = 0.f;
            if (mu < P) {
                const float2 a0 = sacc[mu];
                DF y = {a0.x, a0.y};
                for (int e = combptr[mu]; e < combptr[mu + 1]; ++e) df_fma(y, combg[e], sacc[combq[e]]);
                // r = b - y
                const float2 bv = brow[mu];
                const DF s = two_sum(bv.x, -y.h);
                rv = __fadd_rn(s.h, __fadd_rn(s.l, __fsub_rn(bv.y, y.l)));
            }
            rrow[mu] = rv;
            acc_t = __fmaf_rn(rv, rv, acc_t);
        }
        __syncwarp();
    }
    double acc = (double)acc_t;
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if (lane == 0) red[warp] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int w = 0; w < DWPB; ++w) s += red[w];
        partials[blockIdx.x] = s;
    }
}

template <int QT>
int launch_df(sgfem_context* ctx, const float2* xs, const float2* bs, float* r32, double* partials, int grid) {
    const size_t smem = (size_t)(2 * ctx->ld + ctx->M1 + 1 + ctx->Qn) * sizeof(float2) * DWPB;
    if (grid == 0) {
        if (smem > 48 * 1024)
            SG_CUDA(ctx, cudaFuncSetAttribute(k_residual_df<QT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        return SGFEM_OK;
    }
    k_residual_df<QT><<<grid, DWPB * 32, smem, ctx->stream>>>(
        ctx->d_rowptr, ctx->d_col, (const float2*)ctx->d_valdf, ctx->M1, xs, bs, r32, (int)ctx->n, (int)ctx->P,
        (int)ctx->ld, ctx->d_bmask, ctx->d_qtab, ctx->Qn, ctx->d_combptr, ctx->d_combq,
        (const float2*)ctx->d_combgdf, ctx->rowsum_zero ? 1 : 0, partials);
    SG_LAUNCHED(ctx);
    return SGFEM_OK;
}

int launch_df_qt(sgfem_context* ctx, const float2* xs, const float2* bs, float* r32, double* partials, int grid) {
    const int need = (ctx->Qn + 31) / 32;
    if (need <= 4) return launch_df<4>(ctx, xs, bs, r32, partials, grid);
    if (need <= 8) return launch_df<8>(ctx, xs, bs, r32, partials, grid);
    if (need <= 12) return launch_df<12>(ctx, xs, bs, r32, partials, grid);
    if (need <= 16) return launch_df<16>(ctx, xs, bs, r32, partials, grid);
    if (need <= 20) return launch_df<20>(ctx, xs, bs, r32, partials, grid);
    return launch_df<24>(ctx, xs, bs, r32, partials, grid);  // rounds for larger Q
}

}  // namespace

bool sg_residual_df_usable(const sgfem_context* ctx) {
    // one KLE value per lane is staged per nonzero: M + 1 <= 32 terms
    if (ctx->batched || !ctx->rowsum_zero || ctx->Qn <= 0 || ctx->M1 > 32) return false;
    const size_t smem = (size_t)(2 * ctx->ld + ctx->M1 + 1 + ctx->Qn) * sizeof(float2) * DWPB;
    if (smem > 200 * 1024) return false;
    const char* e = getenv("SGFEM_RESIDUAL");
    return !(e && std::string(e) == "fp64");
}

int sg_residual_df_prepare(sgfem_context* ctx) {
    if (ctx->d_valdf && ctx->d_combgdf) return SGFEM_OK;
    const int grid = ctx->num_sms * 8;
    if (!ctx->d_valdf) {  // the K_m (kept across coupling updates)
        const size_t nv = (size_t)ctx->nnz * ctx->M1;
        SG_CUDA(ctx, cudaMalloc(&ctx->d_valdf, nv * sizeof(float2)));
        k_split_pairs<<<grid, 256, 0, ctx->stream>>>(ctx->d_val64, (float2*)ctx->d_valdf, nv);
        SG_LAUNCHED(ctx);
    }
    SG_CUDA(ctx, cudaMalloc(&ctx->d_combgdf, std::max<size_t>(1, (size_t)ctx->ncomb) * sizeof(float2)));
    if (ctx->ncomb > 0) {
        k_split_pairs<<<grid, 256, 0, ctx->stream>>>(ctx->d_combg64, (float2*)ctx->d_combgdf, (size_t)ctx->ncomb);
        SG_LAUNCHED(ctx);
    }
    SG_TRY(launch_df_qt(ctx, nullptr, nullptr, nullptr, nullptr, 0));
    return SGFEM_OK;
}

int sg_split_df(sgfem_context* ctx, double* x, const double* d, void* xs, int add) {
    const size_t total = (size_t)ctx->n * ctx->ld;
    const int grid = (int)std::min<int64_t>((int64_t)((total + 255) / 256), (int64_t)ctx->num_sms * 8);
    k_add_split<<<grid, 256, 0, ctx->stream>>>(x, d, (float2*)xs, total, add);
    SG_LAUNCHED(ctx);
    return SGFEM_OK;
}

int sg_residual_df(sgfem_context* ctx, const void* xs, const void* bs, float* r32, double* partials, int* nblocks) {
    int grid = (int)std::min<int64_t>((ctx->n + DWPB - 1) / DWPB, (int64_t)ctx->num_sms * 8);
    if (grid < 1) grid = 1;
    if (nblocks) *nblocks = grid;
    return launch_df_qt(ctx, (const float2*)xs, (const float2*)bs, r32, partials, grid);
}

extern "C" int sgfem_time_residual(sgfem_context* ctx, int reps, double* ms_per_residual, int* kind) {
    SG_TRY(sg_check_ready(ctx));
    if (reps <= 0 || !ms_per_residual) return sg_fail(ctx, SGFEM_ERR_ARGUMENT, "bad reps");
    if (ctx->batched) return sg_fail(ctx, SGFEM_ERR_STATE, "sgfem_time_residual: samples context");
    SG_CUDA(ctx, cudaSetDevice(ctx->device));
    const bool df = sg_residual_df_usable(ctx);
    if (kind) *kind = df ? 1 : 0;
    const size_t total = (size_t)ctx->n * ctx->ld, n64 = total * sizeof(double);
    for (int i : {0, 1, 12, 13}) SG_TRY(sg_ensure(ctx, ctx->w_vec[i], n64));
    SG_TRY(sg_ensure(ctx, ctx->w_partials, (size_t)(ctx->num_sms * 8 + 8) * sizeof(double)));
    void* xs = ctx->w_vec[12].p;
    void* bs = ctx->w_vec[13].p;
    float* r32 = (float*)ctx->w_vec[1].p;
    double* partials = (double*)ctx->w_partials.p;
    SG_CUDA(ctx, cudaMemsetAsync(xs, 0, n64, ctx->stream));
    SG_CUDA(ctx, cudaMemsetAsync(bs, 0, n64, ctx->stream));
    SG_CUDA(ctx, cudaMemsetAsync(ctx->w_vec[0].p, 0, n64, ctx->stream));
    if (df) SG_TRY(sg_residual_df_prepare(ctx));
    auto one = [&]() -> int {
        if (df) return sg_residual_df(ctx, xs, bs, r32, partials, nullptr);
        return sg_launch_apply(ctx, SGFEM_FP64, ctx->w_vec[0].p, xs, partials, nullptr, nullptr);
    };
    SG_TRY(one());
    SG_CUDA(ctx, cudaEventRecord(ctx->ev0, ctx->stream));
    for (int r = 0; r < reps; ++r) SG_TRY(one());
    SG_CUDA(ctx, cudaEventRecord(ctx->ev1, ctx->stream));
    SG_CUDA(ctx, cudaEventSynchronize(ctx->ev1));
    float ms = 0.f;
    SG_CUDA(ctx, cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
    *ms_per_residual = ms / reps;
    return SGFEM_OK;
}
