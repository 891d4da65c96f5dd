// K3b: restarted GMRES on the device for SG operators that are not symmetric.
//
// Replaces solve_logpoisson_primal! (src/modelproblems/solvers_logpoisson_primal.jl:130-172),
// whose operator Y_mu = (A + N_0) X_mu + sum_{m,nu} G[(m-1)P+mu, nu] N_m X_nu has the
// non-symmetric convection blocks N_m = -(grad a_m . grad u, v).  The reference calls
// Krylov.gmres with the mean-based preconditioner as a left preconditioner; here GMRES is
// right-preconditioned, so its residual estimate is the unpreconditioned residual and the
// stop test is the FP64 true residual ||b - A x|| <= rtol ||b|| (the same test as the
// symmetric solver).  Both converge to the same solution.
//
// One Arnoldi step: z = B v_k (mean-based preconditioner), w = A z, classical Gram-Schmidt
// run twice (CGS2) against v_0..v_k with one multi-dot kernel per pass (each block reads
// its slice of w once for eight basis vectors), ||w||, v_{k+1} = w / ||w||.  The
// Hessenberg column, its Givens rotations and the triangular solve are O(restart^2) and run
// on the host from the reduced values.  Reductions are per-block FP64 partials summed in a
// fixed order: results are bitwise reproducible.
// SGFEM_MIXED: FP64 x, b and true residual; each refinement step solves A d = r with
// FP32 GMRES (FP32 operator, preconditioner and basis; FP64 dots) to inner_rtol.
#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

#include "sgfem_internal.h"

namespace {

constexpr int GT = 256;    // threads of the vector kernels
constexpr int KMAX = 128;  // largest restart + 1

template <typename T>
__global__ void __launch_bounds__(GT) k_mdot(const T* __restrict__ V, size_t total, int k, const T* __restrict__ w,
                                             double* __restrict__ partials, const KrylovScalars* __restrict__ scal) {
    if (scal && scal->done) return;
    __shared__ double red[GT / 32][8];
    const int i0 = blockIdx.y * 8;
    // per-thread partials in the vectors' precision (GB300's FP64 rate is 1/64 of
    // FP32), block and grid sums in FP64
    T acc[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) acc[i] = T(0);
    for (size_t t = (size_t)blockIdx.x * GT + threadIdx.x; t < total; t += (size_t)gridDim.x * GT) {
        const T wv = w[t];
#pragma unroll
        for (int i = 0; i < 8; ++i)
            if (i0 + i < k) acc[i] = fma(V[(size_t)(i0 + i) * total + t], wv, acc[i]);
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        double a = (double)acc[i];
        for (int o = 16; o > 0; o >>= 1) a += __shfl_down_sync(0xffffffffu, a, o);
        if (lane == 0) red[warp][i] = a;
    }
    __syncthreads();
    if (threadIdx.x < 8 && i0 + (int)threadIdx.x < k) {
        double s = 0.0;
        for (int w2 = 0; w2 < GT / 32; ++w2) s += red[w2][threadIdx.x];
        partials[(size_t)(i0 + threadIdx.x) * gridDim.x + blockIdx.x] = s;
    }
}

// h[i] = sum_b partials[i * nb + b] (fixed order), one block per i
__global__ void __launch_bounds__(GT) k_mdot_fin(const double* __restrict__ partials, int nb, double* __restrict__ h) {
    __shared__ double red[GT];
    double v = 0.0;
    for (int b = threadIdx.x; b < nb; b += GT) v += partials[(size_t)blockIdx.x * nb + b];
    red[threadIdx.x] = v;
    __syncthreads();
    for (int w = GT / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) h[blockIdx.x] = red[0];
}

// device-side Arnoldi bookkeeping: the step's Hessenberg column, the rotations,
// the residual estimate and the stop flag live in device memory, so a step needs
// no host round trip (the host reads the state every few steps)
struct ArnState {
    double res;      // |g[k+1]| after the last completed step
    double inv_nrm;  // 1 / ||w|| of the last step (scales the next basis vector)
    int kk;          // completed steps of this cycle
    int flag;        // 0 running, 1 converged or happy breakdown, 2 singular, 3 non-finite
};

// hneg[i] = -sum_b partials[i * nb + b]; hcol[i] (+)= the sum (CGS2 accumulates both rounds)
__global__ void __launch_bounds__(GT) k_mdot_fin_neg(const double* __restrict__ partials, int nb, double* __restrict__ hneg,
                                                     double* __restrict__ hcol, int accumulate,
                                                     const KrylovScalars* __restrict__ scal) {
    if (scal->done) return;
    __shared__ double red[GT];
    double v = 0.0;
    for (int b = threadIdx.x; b < nb; b += GT) v += partials[(size_t)blockIdx.x * nb + b];
    red[threadIdx.x] = v;
    __syncthreads();
    for (int w = GT / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        hneg[blockIdx.x] = -red[0];
        hcol[blockIdx.x] = accumulate ? hcol[blockIdx.x] + red[0] : red[0];
    }
}

// one thread: column k of the Hessenberg matrix from hcol and ||w||^2 = *nrm2,
// rotations of the earlier steps, the new rotation, the residual estimate
__global__ void k_givens(int k, const double* __restrict__ hcol, const double* __restrict__ nrm2, double* __restrict__ H,
                         int ldh, double* __restrict__ cs, double* __restrict__ sn, double* __restrict__ g,
                         ArnState* __restrict__ st, KrylovScalars* __restrict__ scal, double tol_abs) {
    if (scal->done) return;
    const double nrm = sqrt(*nrm2);
    double* col = H + (size_t)k * ldh;
    for (int i = 0; i <= k; ++i) col[i] = hcol[i];
    for (int i = 0; i < k; ++i) {
        const double a = col[i], c2 = col[i + 1];
        col[i] = cs[i] * a + sn[i] * c2;
        col[i + 1] = -sn[i] * a + cs[i] * c2;
    }
    const double r = hypot(col[k], nrm);
    if (!isfinite(r)) {
        st->flag = 3;
        scal->done = 1;
        return;
    }
    if (r == 0.0) {
        st->flag = 2;
        scal->done = 1;
        return;
    }
    cs[k] = col[k] / r;
    sn[k] = nrm / r;
    col[k] = r;
    col[k + 1] = 0.0;
    g[k + 1] = -sn[k] * g[k];
    g[k] = cs[k] * g[k];
    st->res = fabs(g[k + 1]);
    st->kk = k + 1;
    st->inv_nrm = nrm > 0.0 ? 1.0 / nrm : 0.0;
    if (st->res <= tol_abs || nrm == 0.0) {
        st->flag = 1;
        scal->done = 1;
    }
}

template <typename T>
__global__ void __launch_bounds__(GT) k_scale_dev(T* __restrict__ dst, const T* __restrict__ src, size_t total,
                                                  const ArnState* __restrict__ st, const KrylovScalars* __restrict__ scal) {
    if (scal->done) return;
    const double s = st->inv_nrm;
    for (size_t t = (size_t)blockIdx.x * GT + threadIdx.x; t < total; t += (size_t)gridDim.x * GT)
        dst[t] = (T)((double)src[t] * s);
}

// w = beta * w + sum_i c_i V_i   (beta = 0: w = V c)
template <typename T>
__global__ void __launch_bounds__(GT) k_lincomb(T* __restrict__ w, const T* __restrict__ V, size_t total, int k,
                                                const double* __restrict__ c, double beta,
                                                const KrylovScalars* __restrict__ scal = nullptr) {
    if (scal && scal->done) return;
    __shared__ T cs[KMAX];  // coefficients in the vectors' precision
    for (int i = threadIdx.x; i < k; i += GT) cs[i] = (T)c[i];
    __syncthreads();
    const T bt = (T)beta;
    for (size_t t = (size_t)blockIdx.x * GT + threadIdx.x; t < total; t += (size_t)gridDim.x * GT) {
        T a = beta == 0.0 ? T(0) : bt * w[t];
        for (int i = 0; i < k; ++i) a = fma(cs[i], V[(size_t)i * total + t], a);
        w[t] = a;
    }
}

// x64 += sum_i c_i Z_i (FP64 accumulation of FP32 vectors)
template <typename T>
__global__ void __launch_bounds__(GT) k_lincomb_add64(double* __restrict__ x, const T* __restrict__ Z, size_t total,
                                                      int k, const double* __restrict__ c) {
    __shared__ double cs[KMAX];
    for (int i = threadIdx.x; i < k; i += GT) cs[i] = c[i];
    __syncthreads();
    for (size_t t = (size_t)blockIdx.x * GT + threadIdx.x; t < total; t += (size_t)gridDim.x * GT) {
        double a = x[t];
        for (int i = 0; i < k; ++i) a = fma(cs[i], (double)Z[(size_t)i * total + t], a);
        x[t] = a;
    }
}

template <typename T>
__global__ void __launch_bounds__(GT) k_scale(T* __restrict__ dst, const T* __restrict__ src, size_t total, double s) {
    for (size_t t = (size_t)blockIdx.x * GT + threadIdx.x; t < total; t += (size_t)gridDim.x * GT)
        dst[t] = (T)((double)src[t] * s);
}

// r = b - ax
template <typename T>
__global__ void __launch_bounds__(GT) k_sub(T* __restrict__ r, const T* __restrict__ b, const T* __restrict__ ax,
                                            size_t total) {
    for (size_t t = (size_t)blockIdx.x * GT + threadIdx.x; t < total; t += (size_t)gridDim.x * GT) r[t] = b[t] - ax[t];
}

// x += z
template <typename T, typename U>
__global__ void __launch_bounds__(GT) k_add(T* __restrict__ x, const U* __restrict__ z, size_t total) {
    for (size_t t = (size_t)blockIdx.x * GT + threadIdx.x; t < total; t += (size_t)gridDim.x * GT)
        x[t] = (T)((double)x[t] + (double)z[t]);
}

__global__ void __launch_bounds__(GT) k_demote(float* __restrict__ dst, const double* __restrict__ src, size_t total) {
    for (size_t t = (size_t)blockIdx.x * GT + threadIdx.x; t < total; t += (size_t)gridDim.x * GT) dst[t] = (float)src[t];
}

// b = b0 (device layout) + (x0 if use_x0), Dirichlet rows zeroed
__global__ void __launch_bounds__(GT) k_rhs_full(double* __restrict__ b, const double* __restrict__ x0,
                                                 const unsigned char* __restrict__ bmask, size_t total, int ld,
                                                 int use_x0) {
    for (size_t t = (size_t)blockIdx.x * GT + threadIdx.x; t < total; t += (size_t)gridDim.x * GT) {
        const size_t row = t / ld;
        b[t] = bmask[row] ? 0.0 : (use_x0 ? b[t] + x0[t] : b[t]);
    }
}

struct Gm {
    sgfem_context* ctx;
    int prec_kind;
    size_t total;
    int nbx;
    double* d_part;  // KMAX * nbx
    double* d_h;     // KMAX
    int grid;
    long long applies64 = 0;

    template <typename T>
    int dots(const T* V, int k, const T* w, double* out) {
        dim3 g((unsigned)nbx, (unsigned)((k + 7) / 8));
        k_mdot<T><<<g, GT, 0, ctx->stream>>>(V, total, k, w, d_part, nullptr);
        SG_LAUNCHED(ctx);
        k_mdot_fin<<<k, GT, 0, ctx->stream>>>(d_part, nbx, d_h);
        SG_LAUNCHED(ctx);
        SG_CUDA(ctx, cudaMemcpyAsync(out, d_h, (size_t)k * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
        SG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        return SGFEM_OK;
    }

    template <typename T>
    int norm(const T* v, double* out) {
        double s = 0.0;
        SG_TRY(dots<T>(v, 1, v, &s));
        *out = std::sqrt(s);
        return SGFEM_OK;
    }

    // z = B v (z's Dirichlet rows are left as they are: zero)
    template <typename T>
    int precond(int precision, const T* v, T* z, T* tmp, const KrylovScalars* scal = nullptr) {
        if (prec_kind == SGFEM_PREC_LATTICE) {
            SG_TRY(sg_lat_pass_x(ctx, precision, v, tmp, scal));
            SG_TRY(sg_lat_pass_y(ctx, precision, tmp, nullptr, nullptr, scal));
            return sg_lat_pass_xinv(ctx, precision, tmp, z, 0, scal);
        }
        if (prec_kind == SGFEM_PREC_CHOLESKY) return sg_chol_apply(ctx, precision, v, z, scal);
        return sg_jacobi(ctx, precision, v, z, 0, prec_kind == SGFEM_PREC_NONE ? 1 : 0, nullptr, nullptr, scal);
    }

    template <typename T>
    int apply(int precision, const T* x, T* y, const KrylovScalars* scal = nullptr) {
        if (precision == SGFEM_FP64) applies64++;
        return sg_launch_apply(ctx, precision, x, y, nullptr, nullptr, scal);
    }

    // Restarted right-preconditioned GMRES on A x = b in precision T.  x holds the
    // start (x_zero: zero); stops when ||b - A x|| <= tol_abs (true residual in
    // precision T, FP64 sums) or after maxit Arnoldi steps.  z's Dirichlet rows zero.
    // Flexible form (Z != nullptr, one cycle from a zero start): the preconditioned
    // basis vectors z_k are kept and the cycle ends with x64 += Z y in FP64, so the
    // correction is exactly the combination the Arnoldi relation A Z = V H holds for
    // (x = B (V y) recomputed in FP32 differs from Z y by rough rounding errors that
    // A amplifies by its condition number); *res is the GMRES residual estimate.
    template <typename T>
    int run(int precision, T* x, const T* b, T* V, T* z, T* w, T* tmp, int restart, double tol_abs, int maxit,
            bool x_zero, int* iters, double* res, T* Z = nullptr, double* x64 = nullptr) {
        T* v0 = V;
        if (x_zero) {
            SG_CUDA(ctx, cudaMemcpyAsync(v0, b, total * sizeof(T), cudaMemcpyDeviceToDevice, ctx->stream));
        } else {
            SG_TRY(apply<T>(precision, x, w));
            k_sub<T><<<grid, GT, 0, ctx->stream>>>(v0, b, w, total);
            SG_LAUNCHED(ctx);
        }
        double beta = 0.0;
        SG_TRY(norm<T>(v0, &beta));
        *res = beta;
        *iters = 0;
        if (!std::isfinite(beta)) return sg_fail(ctx, SGFEM_ERR_NONFINITE, "non-finite residual");
        if (beta <= tol_abs) return SGFEM_OK;
        const int m = restart;
        std::vector<double> H((size_t)(m + 1) * m, 0.0), g(m + 1), y(m);
        auto Hat = [&](int i, int j) -> double& { return H[(size_t)j * (m + 1) + i]; };
        // device state of the Arnoldi steps
        KrylovScalars* scal = ctx->d_scal;
        double* d_hcol = d_h + KMAX;
        double* d_H = d_hcol + KMAX;
        double* d_cs = d_H + (size_t)(KMAX + 1) * KMAX;
        double* d_sn = d_cs + KMAX;
        double* d_g = d_sn + KMAX;
        double* d_nrm2 = d_g + KMAX + 1;
        ArnState* d_st = reinterpret_cast<ArnState*>(d_nrm2 + 1);
        constexpr int CHK = 4;  // steps between host checks of the stop flag
        int it = 0;
        for (;;) {
            k_scale<T><<<grid, GT, 0, ctx->stream>>>(v0, v0, total, 1.0 / beta);
            SG_LAUNCHED(ctx);
            std::fill(g.begin(), g.end(), 0.0);
            g[0] = beta;
            ArnState hs{beta, 0.0, 0, 0};
            SG_CUDA(ctx, cudaMemcpyAsync(d_g, g.data(), (size_t)(m + 1) * sizeof(double), cudaMemcpyHostToDevice,
                                         ctx->stream));
            SG_CUDA(ctx, cudaMemcpyAsync(d_st, &hs, sizeof(ArnState), cudaMemcpyHostToDevice, ctx->stream));
            SG_CUDA(ctx, cudaMemsetAsync(scal, 0, sizeof(KrylovScalars), ctx->stream));
            const int kmax = std::min(m, maxit - it);
            for (int k = 0; k < kmax; ++k) {
                T* vk = V + (size_t)k * total;
                T* vn = V + (size_t)(k + 1) * total;
                T* zk = Z ? Z + (size_t)k * total : z;
                SG_TRY(precond<T>(precision, vk, zk, tmp, scal));
                SG_TRY(apply<T>(precision, zk, w, scal));
                // CGS2: twice w -= V (V^T w), the column accumulating both projections
                for (int round = 0; round < 2; ++round) {
                    dim3 gd((unsigned)nbx, (unsigned)((k + 1 + 7) / 8));
                    k_mdot<T><<<gd, GT, 0, ctx->stream>>>(V, total, k + 1, w, d_part, scal);
                    SG_LAUNCHED(ctx);
                    k_mdot_fin_neg<<<k + 1, GT, 0, ctx->stream>>>(d_part, nbx, d_h, d_hcol, round, scal);
                    SG_LAUNCHED(ctx);
                    k_lincomb<T><<<grid, GT, 0, ctx->stream>>>(w, V, total, k + 1, d_h, 1.0, scal);
                    SG_LAUNCHED(ctx);
                }
                k_mdot<T><<<dim3((unsigned)nbx, 1), GT, 0, ctx->stream>>>(w, total, 1, w, d_part, scal);
                SG_LAUNCHED(ctx);
                k_mdot_fin<<<1, GT, 0, ctx->stream>>>(d_part, nbx, d_nrm2);
                SG_LAUNCHED(ctx);
                k_givens<<<1, 1, 0, ctx->stream>>>(k, d_hcol, d_nrm2, d_H, m + 1, d_cs, d_sn, d_g, d_st, scal, tol_abs);
                SG_LAUNCHED(ctx);
                k_scale_dev<T><<<grid, GT, 0, ctx->stream>>>(vn, w, total, d_st, scal);
                SG_LAUNCHED(ctx);
                if ((k + 1) % CHK == 0 || k + 1 == kmax) {
                    SG_CUDA(ctx, cudaMemcpyAsync(&hs, d_st, sizeof(ArnState), cudaMemcpyDeviceToHost, ctx->stream));
                    SG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
                    if (hs.flag) break;
                }
            }
            if (hs.flag == 2) return sg_fail(ctx, SGFEM_ERR_BREAKDOWN, "GMRES breakdown (singular Hessenberg column)");
            if (hs.flag == 3) return sg_fail(ctx, SGFEM_ERR_NONFINITE, "non-finite value in a GMRES iterate");
            const int kk = hs.kk;
            it += kk;
            if (kk == 0) {
                *iters = it;
                return SGFEM_ERR_MAXIT;
            }
            SG_CUDA(ctx, cudaMemcpyAsync(H.data(), d_H, (size_t)(m + 1) * kk * sizeof(double), cudaMemcpyDeviceToHost,
                                         ctx->stream));
            SG_CUDA(ctx, cudaMemcpyAsync(g.data(), d_g, (size_t)(kk + 1) * sizeof(double), cudaMemcpyDeviceToHost,
                                         ctx->stream));
            SG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
            // y = H^-1 g, x += B (V y)
            for (int i = kk - 1; i >= 0; --i) {
                double s = g[i];
                for (int j = i + 1; j < kk; ++j) s -= Hat(i, j) * y[j];
                y[i] = s / Hat(i, i);
            }
            SG_CUDA(ctx, cudaMemcpyAsync(d_h, y.data(), (size_t)kk * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
            if (Z) {
                k_lincomb_add64<T><<<grid, GT, 0, ctx->stream>>>(x64, Z, total, kk, d_h);
                SG_LAUNCHED(ctx);
                *res = std::fabs(g[kk]);
                *iters = it;
                return SGFEM_OK;
            }
            k_lincomb<T><<<grid, GT, 0, ctx->stream>>>(w, V, total, kk, d_h, 0.0);
            SG_LAUNCHED(ctx);
            SG_TRY(precond<T>(precision, w, z, tmp));
            k_add<T, T><<<grid, GT, 0, ctx->stream>>>(x, z, total);
            SG_LAUNCHED(ctx);
            // true residual
            SG_TRY(apply<T>(precision, x, w));
            k_sub<T><<<grid, GT, 0, ctx->stream>>>(v0, b, w, total);
            SG_LAUNCHED(ctx);
            SG_TRY(norm<T>(v0, &beta));
            *res = beta;
            *iters = it;
            if (!std::isfinite(beta)) return sg_fail(ctx, SGFEM_ERR_NONFINITE, "non-finite residual");
            if (beta <= tol_abs) return SGFEM_OK;
            if (it >= maxit) return SGFEM_ERR_MAXIT;
        }
    }
};

}  // namespace

extern "C" int sgfem_solve_gmres(sgfem_context* ctx, const double* b0, double* x_inout, const sgfem_solve_options* opts,
                                 int restart, sgfem_solve_stats* stats) {
    SG_TRY(sg_check_ready(ctx));
    if (!b0 || !x_inout) return sg_fail(ctx, SGFEM_ERR_ARGUMENT, "null pointer");
    if (ctx->batched) return sg_fail(ctx, SGFEM_ERR_STATE, "sgfem_solve_gmres: samples context (use sgfem_solve_samples)");
    sgfem_solve_options o;
    if (opts) o = *opts; else sgfem_default_options(&o);
    if (restart <= 0) restart = 20;
    if (restart > KMAX - 1) return sg_fail(ctx, SGFEM_ERR_ARGUMENT, "restart too large (<= 127)");
    if (o.precision != SGFEM_FP64 && o.precision != SGFEM_MIXED && o.precision != SGFEM_FP32)
        return sg_fail(ctx, SGFEM_ERR_ARGUMENT, "bad precision");
    if (o.preconditioner == SGFEM_PREC_LATTICE && !ctx->lattice)
        return sg_fail(ctx, SGFEM_ERR_UNSUPPORTED, "lattice preconditioner unavailable (dofs do not form a power-of-two lattice)");
    if (o.preconditioner != SGFEM_PREC_LATTICE && o.preconditioner != SGFEM_PREC_JACOBI && o.preconditioner != SGFEM_PREC_NONE &&
        o.preconditioner != SGFEM_PREC_CHOLESKY)
        return sg_fail(ctx, SGFEM_ERR_ARGUMENT, "bad preconditioner kind");
    if (!(o.rtol > 0.0) || o.maxit <= 0) return sg_fail(ctx, SGFEM_ERR_ARGUMENT, "rtol must be > 0 and maxit > 0");
    SG_CUDA(ctx, cudaSetDevice(ctx->device));
    if (o.preconditioner == SGFEM_PREC_CHOLESKY) {
        SG_TRY(sg_chol_ensure(ctx));
        SG_TRY(sg_chol_workspace(ctx, SGFEM_FP64));
    }
    ctx->samples_x_valid = false;
    const size_t total = (size_t)ctx->n * ctx->ld;
    const size_t n64 = total * sizeof(double), n32 = total * sizeof(float);
    const bool low = o.precision != SGFEM_FP64;
    const size_t esz = low ? sizeof(float) : sizeof(double);
    for (int i = 0; i < 4; ++i) SG_TRY(sg_ensure(ctx, ctx->w_vec[i], n64));
    SG_TRY(sg_ensure(ctx, ctx->w_vec[10], n64));
    if (low) {
        for (int i = 5; i < 10; ++i) SG_TRY(sg_ensure(ctx, ctx->w_vec[i], n32));
        SG_TRY(sg_jit_ensure(ctx));
    }
    SG_TRY(sg_ensure(ctx, ctx->w_basis, (size_t)(restart + 1) * total * esz));
    if (low) SG_TRY(sg_ensure(ctx, ctx->w_zbasis, (size_t)restart * total * sizeof(float)));
    const int grid = (int)std::max<int64_t>(1, std::min<int64_t>((int64_t)((total + GT * 4 - 1) / (GT * 4)),
                                                                 (int64_t)ctx->num_sms * 8));
    const int nbx = std::min(grid, ctx->num_sms * 4);
    // partials | h | Hessenberg column | H | cs | sn | g | ||w||^2 | Arnoldi state
    SG_TRY(sg_ensure(ctx, ctx->w_gsmall,
                     ((size_t)KMAX * nbx + 2 * KMAX + (size_t)(KMAX + 1) * KMAX + 3 * KMAX + 1 + 1 + 8) * sizeof(double)));
    Gm G{ctx, o.preconditioner, total, nbx, (double*)ctx->w_gsmall.p, (double*)ctx->w_gsmall.p + (size_t)KMAX * nbx,
         grid};

    double* x64 = (double*)ctx->w_vec[10].p;
    double* b64 = (double*)ctx->w_vec[0].p;
    const long long launches0 = ctx->launches;
    SG_TRY(sgfem_to_device_layout(ctx, x_inout, x64, SGFEM_FP64));
    SG_TRY(sgfem_to_device_layout(ctx, b0, b64, SGFEM_FP64));
    SG_CUDA(ctx, cudaEventRecord(ctx->ev0, ctx->stream));
    k_rhs_full<<<grid, GT, 0, ctx->stream>>>(b64, x64, ctx->d_bmask, total, (int)ctx->ld, o.reference_rhs ? 1 : 0);
    SG_LAUNCHED(ctx);
    double bnorm = 0.0;
    SG_TRY(G.norm<double>(b64, &bnorm));
    sgfem_solve_stats st{};
    st.apply_ms = -1.0;
    st.precond_ms = -1.0;
    int status = SGFEM_OK;
    if (!std::isfinite(bnorm)) return sg_fail(ctx, SGFEM_ERR_NONFINITE, "non-finite right-hand side");
    const double tol = o.rtol * bnorm;
    if (bnorm == 0.0) {
        SG_CUDA(ctx, cudaMemsetAsync(x64, 0, n64, ctx->stream));
        st.relres = 0.0;
    } else if (!low) {
        double* z = (double*)ctx->w_vec[1].p;
        double* w = (double*)ctx->w_vec[2].p;
        double* tmp = (double*)ctx->w_vec[3].p;
        SG_CUDA(ctx, cudaMemsetAsync(z, 0, n64, ctx->stream));
        int its = 0;
        double res = 0.0;
        status = G.run<double>(SGFEM_FP64, x64, b64, (double*)ctx->w_basis.p, z, w, tmp, restart, tol, o.maxit, false,
                               &its, &res);
        if (status != SGFEM_OK && status != SGFEM_ERR_MAXIT) return status;
        st.iterations = its;
        st.outer_iterations = 1;
        st.relres = res / bnorm;
    } else {
        // FP64 refinement around FP32 GMRES
        double* r64 = (double*)ctx->w_vec[1].p;
        double* t64 = (double*)ctx->w_vec[2].p;
        float* b32 = (float*)ctx->w_vec[5].p;
        float* d32 = (float*)ctx->w_vec[6].p;
        float* z32 = (float*)ctx->w_vec[7].p;
        float* w32 = (float*)ctx->w_vec[8].p;
        float* tmp32 = (float*)ctx->w_vec[9].p;
        float* V32 = (float*)ctx->w_basis.p;
        SG_CUDA(ctx, cudaMemsetAsync(z32, 0, n32, ctx->stream));
        int total_it = 0, outer = 0;
        double res = 0.0;
        for (;;) {
            SG_TRY(G.apply<double>(SGFEM_FP64, x64, t64));
            k_sub<double><<<grid, GT, 0, ctx->stream>>>(r64, b64, t64, total);
            SG_LAUNCHED(ctx);
            SG_TRY(G.norm<double>(r64, &res));
            if (!std::isfinite(res)) return sg_fail(ctx, SGFEM_ERR_NONFINITE, "non-finite residual");
            if (res <= tol) break;
            if (total_it >= o.maxit || outer >= 200) {
                status = SGFEM_ERR_MAXIT;
                break;
            }
            if (o.precision == SGFEM_FP32 && outer > 0) break;  // plain FP32 solve: one pass
            k_demote<<<grid, GT, 0, ctx->stream>>>(b32, r64, total);
            SG_LAUNCHED(ctx);
            int its = 0;
            double rin = 0.0;
            int rc;
            if (o.precision == SGFEM_FP32) {
                SG_CUDA(ctx, cudaMemsetAsync(d32, 0, n32, ctx->stream));
                rc = G.run<float>(SGFEM_FP32, d32, b32, V32, z32, w32, tmp32, restart, o.rtol * res, o.maxit - total_it,
                                  true, &its, &rin);
                if (rc != SGFEM_OK && rc != SGFEM_ERR_MAXIT) return rc;
                k_add<double, float><<<grid, GT, 0, ctx->stream>>>(x64, d32, total);
                SG_LAUNCHED(ctx);
            } else {
                // one flexible FP32 cycle per refinement step, its correction accumulated in
                // FP64; first step to inner_rtol, later steps aim to end the solve (margin 3,
                // at most a 1e-6 reduction per cycle)
                const double finish = 0.3 * tol / res;
                const double inner = outer == 0 ? std::max(o.inner_rtol, finish) : std::max(finish, 1e-6);
                rc = G.run<float>(SGFEM_FP32, d32, b32, V32, z32, w32, tmp32, restart, inner * res,
                                  std::min(restart, o.maxit - total_it), true, &its, &rin,
                                  (float*)ctx->w_zbasis.p, x64);
                if (rc != SGFEM_OK && rc != SGFEM_ERR_MAXIT) return rc;
            }
            total_it += its;
            ++outer;
            if (its == 0) {  // FP32 cannot reduce the residual further
                status = SGFEM_ERR_MAXIT;
                break;
            }
        }
        st.iterations = total_it;
        st.outer_iterations = outer;
        st.relres = res / bnorm;
        if (o.precision == SGFEM_FP32 && status == SGFEM_OK && st.relres > o.rtol) status = SGFEM_ERR_MAXIT;
    }
    SG_CUDA(ctx, cudaEventRecord(ctx->ev1, ctx->stream));
    SG_CUDA(ctx, cudaEventSynchronize(ctx->ev1));
    float ms = 0.f;
    SG_CUDA(ctx, cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
    st.time_ms = ms;
    if (low) SG_TRY(sg_jit_check(ctx));
    st.fp64_applies = (int)G.applies64;
    st.kernel_launches = ctx->launches - launches0;
    if (stats) *stats = st;
    SG_TRY(sgfem_from_device_layout(ctx, x64, x_inout, SGFEM_FP64));
    if (status == SGFEM_ERR_MAXIT) return sg_fail(ctx, status, "tolerance not reached within maxit");
    return status;
}
