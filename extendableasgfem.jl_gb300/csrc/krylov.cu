// K3: device-resident preconditioned CG and mixed-precision refinement.
//
// Replaces solve_primal! (src/modelproblems/solvers_poisson_primal.jl:130-169):
//   * right-hand side b = x0 + e_1 (x) b0 with Dirichlet rows zeroed (:149-155),
//     x0 the warm start taken from SGFEVector.entries;
//   * the reference's left-preconditioned GMRES (Krylov.gmres, :160) becomes
//     PCG: the SG operator of PoissonProblemPrimal is symmetric positive
//     definite on interior dofs and the mean-based preconditioner is SPD, so
//     both reach the same solution; PCG needs two inner products per step.
// Iteration (all scalars live in device memory, no host round trip):
//   q = A p (+ p'q partials)      -> finalize: alpha = rho / p'q
//   x += alpha p, r -= alpha q    -> finalize: rr, convergence flag
//   z = B r (three lattice passes, r'z by Parseval) -> finalize: beta
//   p = z + beta p (fused into the last preconditioner pass)
// Reductions are per-block FP64 partials summed by one block in a fixed
// order, so results are bitwise reproducible run to run.  The iterations run
// as a device-side loop (a CUDA graph conditional WHILE node) that stops when
// the convergence flag is set; kernels return immediately once it is.
// SGFEM_MIXED: FP64 x, b and true residual r = b - A x; each refinement step
// solves A d = r with FP32 PCG (FP32 operator values, vectors and
// accumulation; FP64 inner products) to inner_rtol and adds d to x in FP64.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "sgfem_internal.h"

namespace {

constexpr int VT = 256;  // threads of vector kernels

enum FinMode { FIN_ALPHA = 0, FIN_RR = 1, FIN_BETA = 2, FIN_TOL = 3, FIN_SUM = 4 };

struct FinArgs {
    double rtol2;  // FIN_TOL: tol2 = rtol2 * sum
    int maxit;
    int loop;      // 1: last finalize of a device-loop body, sets the loop condition
    cudaGraphConditionalHandle handle;
};

// one finalize step of the PCG scalars; sticky done flag
__device__ void fin_step(KrylovScalars* s, int mode, double sum) {
    if (s->done) return;
    if (mode == FIN_ALPHA) {
        s->pq = sum;
        if (!isfinite(sum)) { s->status = SGFEM_ERR_NONFINITE; s->done = 1; return; }
        if (!(sum > 0.0)) { s->status = SGFEM_ERR_BREAKDOWN; s->done = 1; return; }
        s->alpha = s->rho / sum;
    } else if (mode == FIN_RR) {
        s->rr = sum;
        if (!s->first) s->iters += 1;
        if (!isfinite(sum)) { s->status = SGFEM_ERR_NONFINITE; s->done = 1; return; }
        if (sum <= s->tol2) { s->done = 1; return; }
        if (s->iters >= s->maxit) { s->status = SGFEM_ERR_MAXIT; s->done = 1; return; }
    } else if (mode == FIN_BETA) {
        if (!isfinite(sum)) { s->status = SGFEM_ERR_NONFINITE; s->done = 1; return; }
        if (!(sum > 0.0)) { s->status = SGFEM_ERR_BREAKDOWN; s->done = 1; return; }
        if (s->first) {
            s->beta = 0.0;
            s->first = 0;
        } else {
            s->beta = sum / s->rho;
        }
        s->rho = sum;
    }
}

__global__ void k_finalize(const double* __restrict__ partials, int nb, KrylovScalars* __restrict__ s, int mode,
                           FinArgs fa, double* __restrict__ out_sum) {
    __shared__ double red[VT];
    double v = 0.0;
    for (int i = threadIdx.x; i < nb; i += VT) v += partials[i];
    red[threadIdx.x] = v;
    __syncthreads();
    for (int w = VT / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x != 0) return;
    const double sum = red[0];
    if (mode == FIN_SUM) {
        *out_sum = sum;
        return;
    }
    if (mode == FIN_TOL) {
        s->tol2 = fa.rtol2 * sum;
        if (out_sum) *out_sum = sum;
        return;
    }
    fin_step(s, mode, sum);
    if (fa.loop) {
        // the device loop runs another body while the solve goes on; the body count
        // is capped at maxit + 1 (every body not stopped by the flag is an iteration)
        const int bodies = ++s->loops;
        cudaGraphSetConditional(fa.handle, (!s->done && bodies <= s->maxit + 1) ? 1u : 0u);
    }
}

// scalars of a new PCG run: everything zero but tol2 (set by the caller)
__global__ void k_pcg_reset(KrylovScalars* s, int maxit) {
    const double tol2 = s->tol2;
    *s = KrylovScalars{};
    s->tol2 = tol2;
    s->first = 1;
    s->maxit = maxit;
}

__device__ __forceinline__ void block_partial(double acc, double* partials) {
    __shared__ double red[VT / 32];
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int w = 0; w < VT / 32; ++w) s += red[w];
        partials[blockIdx.x] = s;
    }
}

// x += alpha p ; r -= alpha q ; partial ||r||^2.  TX = double with T = float: the
// solution of an FP32 PCG accumulates in FP64 (stored in FP32 its rounding errors
// are rough vectors that A amplifies by its condition number, ~1/h^2, and the true
// residual then stalls near kappa * 2^-24 whatever the recurrence says)
template <typename T, typename TX = T>
__global__ void __launch_bounds__(VT) k_update(TX* __restrict__ x, const T* __restrict__ p, T* __restrict__ r,
                                               const T* __restrict__ q, size_t total, const KrylovScalars* __restrict__ s,
                                               double* __restrict__ partials) {
    if (s->done) return;
    const T alpha = (T)s->alpha;
    const TX alpha_x = (TX)s->alpha;
    T acc_t = T(0);  // per-thread partial in the working precision (narrow FP64 pipe)
    for (size_t i = (size_t)blockIdx.x * VT + threadIdx.x; i < total; i += (size_t)gridDim.x * VT) {
        x[i] = fma(alpha_x, (TX)p[i], x[i]);
        const T rn = fma(-alpha, q[i], r[i]);
        r[i] = rn;
        acc_t = fma(rn, rn, acc_t);
    }
    block_partial((double)acc_t, partials);
}

// r = b - ax ; partial ||r||^2
__global__ void __launch_bounds__(VT) k_residual(const double* __restrict__ b, const double* __restrict__ ax,
                                                 double* __restrict__ r, size_t total, double* __restrict__ partials) {
    double acc = 0.0;
    for (size_t i = (size_t)blockIdx.x * VT + threadIdx.x; i < total; i += (size_t)gridDim.x * VT) {
        const double v = b[i] - ax[i];
        r[i] = v;
        acc += v * v;
    }
    block_partial(acc, partials);
}

// partial sum of a .* b
template <typename T>
__global__ void __launch_bounds__(VT) k_dot(const T* __restrict__ a, const T* __restrict__ b, size_t total,
                                            double* __restrict__ partials) {
    T acc_t = T(0);
    for (size_t i = (size_t)blockIdx.x * VT + threadIdx.x; i < total; i += (size_t)gridDim.x * VT)
        acc_t = fma(a[i], b[i], acc_t);
    block_partial((double)acc_t, partials);
}

// r32 = (float) r64 ; d32 = 0 ; partial ||r32||^2
__global__ void __launch_bounds__(VT) k_demote(const double* __restrict__ r64, float* __restrict__ r32,
                                               double* __restrict__ d64, size_t total, double* __restrict__ partials) {
    float acc_t = 0.0f;
    for (size_t i = (size_t)blockIdx.x * VT + threadIdx.x; i < total; i += (size_t)gridDim.x * VT) {
        const float v = (float)r64[i];
        r32[i] = v;
        d64[i] = 0.0;
        acc_t = fmaf(v, v, acc_t);
    }
    block_partial((double)acc_t, partials);
}

// partial ||r - q||^2 with r in FP64 and q in FP32 (refinement diagnostics)
__global__ void __launch_bounds__(VT) k_diffnorm(const double* __restrict__ r, const float* __restrict__ q, size_t total,
                                                 double* __restrict__ partials) {
    double acc = 0.0;
    for (size_t i = (size_t)blockIdx.x * VT + threadIdx.x; i < total; i += (size_t)gridDim.x * VT) {
        const double d = r[i] - (double)q[i];
        acc = fma(d, d, acc);
    }
    block_partial(acc, partials);
}

// x64 += d64
__global__ void __launch_bounds__(VT) k_add64(double* __restrict__ x, const double* __restrict__ d, size_t total) {
    for (size_t i = (size_t)blockIdx.x * VT + threadIdx.x; i < total; i += (size_t)gridDim.x * VT) x[i] += d[i];
}

// r64 = (double) r32 (refinement diagnostics)
__global__ void __launch_bounds__(VT) k_to_f64(const float* __restrict__ r, double* __restrict__ o, size_t total) {
    for (size_t i = (size_t)blockIdx.x * VT + threadIdx.x; i < total; i += (size_t)gridDim.x * VT) o[i] = (double)r[i];
}

// d32 = (float) d64 (refinement diagnostics)
__global__ void __launch_bounds__(VT) k_to_f32(const double* __restrict__ d, float* __restrict__ o, size_t total) {
    for (size_t i = (size_t)blockIdx.x * VT + threadIdx.x; i < total; i += (size_t)gridDim.x * VT) o[i] = (float)d[i];
}

// b = (x0 or 0) + e_1 (x) b0, Dirichlet rows zeroed.  b0 in caller order.
__global__ void k_build_rhs(const double* __restrict__ b0, const double* __restrict__ x0, double* __restrict__ b,
                            const int* __restrict__ iperm, const unsigned char* __restrict__ bmask, int n, int ld,
                            int use_x0) {
    const size_t total = (size_t)n * ld;
    for (size_t i = (size_t)blockIdx.x * VT + threadIdx.x; i < total; i += (size_t)gridDim.x * VT) {
        const int row = (int)(i / ld);
        b[i] = (use_x0 && !bmask[row]) ? x0[i] : 0.0;
    }
}

// b0 goes to the device column c0 of caller mode 0 (the column order is permuted)
__global__ void k_add_b0(const double* __restrict__ b0, double* __restrict__ b, const int* __restrict__ iperm,
                         const unsigned char* __restrict__ bmask, int n, int ld, int c0) {
    for (int i = blockIdx.x * VT + threadIdx.x; i < n; i += gridDim.x * VT) {
        const int row = iperm[i];
        if (!bmask[row]) b[(size_t)row * ld + c0] += b0[i];
    }
}

// b[row, s] = b0[caller dof] in every column (sample problems), Dirichlet rows zero
__global__ void k_build_rhs_all(const double* __restrict__ b0, double* __restrict__ b, const int* __restrict__ iperm,
                                const unsigned char* __restrict__ bmask, int n, int S, int ld) {
    const size_t total = (size_t)n * ld;
    for (size_t t = (size_t)blockIdx.x * VT + threadIdx.x; t < total; t += (size_t)gridDim.x * VT) {
        const int i = (int)(t / ld), s = (int)(t - (size_t)i * ld);
        const int row = iperm[i];
        b[(size_t)row * ld + s] = (s < S && !bmask[row]) ? b0[i] : 0.0;
    }
}

// out[s] = sum_i v[i * ld + s]^2, one block per column
__global__ void k_colnorm2(const double* __restrict__ v, int n, int ld, double* __restrict__ out) {
    __shared__ double red[VT];
    double a = 0.0;
    for (int i = threadIdx.x; i < n; i += VT) {
        const double x = v[(size_t)i * ld + blockIdx.x];
        a += x * x;
    }
    red[threadIdx.x] = a;
    __syncthreads();
    for (int w = VT / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) out[blockIdx.x] = red[0];
}

int vgrid(const sgfem_context* ctx) {
    const int64_t total = ctx->n * ctx->ld;
    return (int)std::max<int64_t>(1, std::min<int64_t>((total + VT * 4 - 1) / (VT * 4), (int64_t)ctx->num_sms * 8));
}

struct Solver {
    sgfem_context* ctx;
    int prec_kind;
    double* partials;
    KrylovScalars* s;

    int loop = 0;  // set while the last iteration of a device-loop body is captured
    cudaGraphConditionalHandle loop_handle = 0;

    int fin(int nb, int mode, FinArgs fa = FinArgs{0.0, 0, 0, 0}, double* out = nullptr) {
        if (mode == FIN_BETA && loop) {
            fa.loop = 1;
            fa.handle = loop_handle;
        }
        k_finalize<<<1, VT, 0, ctx->stream>>>(partials, nb, s, mode, fa, out);
        SG_LAUNCHED(ctx);
        return SGFEM_OK;
    }

    // z = B r and p = z + beta p, with rho/beta finalized in between
    template <typename T>
    int precond_block(int precision, T* r, T* p, T* tmp, int maxit) {
        int nb = 0;
        FinArgs fa{0.0, maxit, 0, 0};
        if (prec_kind == SGFEM_PREC_LATTICE) {
            SG_TRY(sg_lat_pass_x(ctx, precision, r, tmp, s));
            SG_TRY(sg_lat_pass_y(ctx, precision, tmp, partials, &nb, s));
            SG_TRY(fin(nb, FIN_BETA, fa));
            SG_TRY(sg_lat_pass_xinv(ctx, precision, tmp, p, 1, s));
        } else if (prec_kind == SGFEM_PREC_CHOLESKY) {
            SG_TRY(sg_chol_apply(ctx, precision, r, tmp, s));
            SG_TRY(sg_chol_finish(ctx, precision, r, tmp, p, 2, partials, &nb, s));
            SG_TRY(fin(nb, FIN_BETA, fa));
            SG_TRY(sg_chol_finish(ctx, precision, r, tmp, p, 1, nullptr, nullptr, s));
        } else {
            const int identity = prec_kind == SGFEM_PREC_NONE ? 1 : 0;
            SG_TRY(sg_jacobi(ctx, precision, r, p, 2, identity, partials, &nb, s));
            SG_TRY(fin(nb, FIN_BETA, fa));
            SG_TRY(sg_jacobi(ctx, precision, r, p, 1, identity, nullptr, nullptr, s));
        }
        return SGFEM_OK;
    }

    template <typename T, typename TX = T>
    int iteration(int precision, TX* x, T* r, T* p, T* q, T* tmp, int maxit) {
        int nb = 0;
        FinArgs fa{0.0, maxit, 0, 0};
        SG_TRY(sg_launch_apply(ctx, precision, p, q, partials, &nb, s));
        SG_TRY(fin(nb, FIN_ALPHA, fa));
        const size_t total = (size_t)ctx->n * ctx->ld;
        const int g = vgrid(ctx);
        k_update<T, TX><<<g, VT, 0, ctx->stream>>>(x, p, r, q, total, s, partials);
        SG_LAUNCHED(ctx);
        SG_TRY(fin(g, FIN_RR, fa));
        SG_TRY(precond_block<T>(precision, r, p, tmp, maxit));
        return SGFEM_OK;
    }

    // PCG on A x = b given r = b - A x on entry, stopping when ||r||^2 <= s->tol2
    // (set by the caller).  Returns the status; iterations in *iters.
    // The iterations run as one CUDA graph launch: a conditional WHILE node whose
    // body is check_every iterations; the last FIN_BETA finalize of the body clears
    // the loop condition once the done flag is set, so the convergence test costs
    // no host round trip and at most check_every - 1 iterations of early returns.
    template <typename T, typename TX = T>
    int pcg(int precision, TX* x, T* r, T* p, T* q, T* tmp, int maxit, int check_every, int* iters) {
        const size_t vb = (size_t)ctx->n * ctx->ld * sizeof(T);
        SG_CUDA(ctx, cudaMemsetAsync(p, 0, vb, ctx->stream));
        k_pcg_reset<<<1, 1, 0, ctx->stream>>>(s, maxit);
        SG_LAUNCHED(ctx);
        const size_t total = (size_t)ctx->n * ctx->ld;
        const int g = vgrid(ctx);
        k_dot<T><<<g, VT, 0, ctx->stream>>>(r, r, total, partials);
        SG_LAUNCHED(ctx);
        SG_TRY(fin(g, FIN_RR, FinArgs{0.0, maxit, 0, 0}));
        SG_TRY(precond_block<T>(precision, r, p, tmp, maxit));

        // SGFEM_PCG_LOOP=host: the graph is check_every plain iterations, replayed by a
        // host loop that reads the scalars between replays (for tools that do not
        // profile the kernels of conditional graph bodies, and drivers without them)
        const char* elp = getenv("SGFEM_PCG_LOOP");
        const bool host_loop = elp && std::strcmp(elp, "host") == 0;
        // the graph depends only on the buffers, the kernel choice and the block
        // counts (the iteration cap lives in the device scalars), so the instantiated
        // graph of the previous run on the same buffers is replayed
        const uint64_t key[13] = {(uint64_t)precision, (uint64_t)sizeof(T), (uint64_t)sizeof(TX), (uint64_t)(uintptr_t)x,
                                  (uint64_t)(uintptr_t)r, (uint64_t)(uintptr_t)p, (uint64_t)(uintptr_t)q,
                                  (uint64_t)(uintptr_t)tmp, (uint64_t)check_every, (uint64_t)prec_kind,
                                  (uint64_t)(uintptr_t)partials, (uint64_t)(uintptr_t)s, (uint64_t)host_loop};
        if (!ctx->pcg_exec || std::memcmp(key, ctx->pcg_key, sizeof(key)) != 0) {
            if (ctx->pcg_exec) cudaGraphExecDestroy(ctx->pcg_exec);
            if (ctx->pcg_graph) cudaGraphDestroy(ctx->pcg_graph);
            ctx->pcg_exec = nullptr;
            ctx->pcg_graph = nullptr;
            cudaGraph_t graph = nullptr;
            SG_CUDA(ctx, cudaGraphCreate(&graph, 0));
            cudaGraph_t body = graph;  // host loop: the iterations are the graph itself
            cudaError_t ce = cudaSuccess;
            cudaGraphConditionalHandle h = 0;
            if (!host_loop) {
                ce = cudaGraphConditionalHandleCreate(&h, graph, 1, cudaGraphCondAssignDefault);
                cudaGraphNodeParams np{};
                np.type = cudaGraphNodeTypeConditional;
                np.conditional.handle = h;
                np.conditional.type = cudaGraphCondTypeWhile;
                np.conditional.size = 1;
                cudaGraphNode_t node = nullptr;
                if (ce == cudaSuccess) ce = cudaGraphAddNode(&node, graph, nullptr, nullptr, 0, &np);
                body = ce == cudaSuccess ? np.conditional.phGraph_out[0] : nullptr;
            }
            if (ce == cudaSuccess)
                ce = cudaStreamBeginCaptureToGraph(ctx->stream, body, nullptr, nullptr, 0,
                                                   cudaStreamCaptureModeThreadLocal);
            if (ce != cudaSuccess) {
                cudaGraphDestroy(graph);
                return sg_cuda_fail(ctx, ce, "PCG device loop");
            }
            int st = SGFEM_OK;
            const long long before = ctx->launches;
            loop_handle = h;
            for (int k = 0; k < check_every && st == SGFEM_OK; ++k) {
                loop = !host_loop && k == check_every - 1;
                st = iteration<T, TX>(precision, x, r, p, q, tmp, maxit);
            }
            loop = 0;
            const long long per_body = ctx->launches - before;  // kernel nodes per loop body
            ctx->launches = before;
            ce = cudaStreamEndCapture(ctx->stream, &body);
            if (st != SGFEM_OK || ce != cudaSuccess) {
                cudaGraphDestroy(graph);
                return st != SGFEM_OK ? st : sg_cuda_fail(ctx, ce, "PCG device loop capture");
            }
            cudaGraphExec_t ex = nullptr;
            cudaError_t ie = cudaGraphInstantiate(&ex, graph, 0);
            if (ie != cudaSuccess) {
                cudaGraphDestroy(graph);
                return sg_cuda_fail(ctx, ie, "cudaGraphInstantiate");
            }
            ctx->pcg_graph = graph;
            ctx->pcg_exec = ex;
            ctx->pcg_per_graph = per_body;
            std::memcpy(ctx->pcg_key, key, sizeof(key));
        }
        const KrylovScalars* hs = ctx->h_scal;
        if (host_loop) {
            for (;;) {
                SG_CUDA(ctx, cudaMemcpyAsync(ctx->h_scal, s, sizeof(KrylovScalars), cudaMemcpyDeviceToHost, ctx->stream));
                SG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
                if (hs->done) break;
                cudaError_t le = cudaGraphLaunch(ctx->pcg_exec, ctx->stream);
                if (le != cudaSuccess) return sg_cuda_fail(ctx, le, "cudaGraphLaunch");
                ctx->launches += ctx->pcg_per_graph;
            }
        } else {
            cudaError_t le = cudaGraphLaunch(ctx->pcg_exec, ctx->stream);
            if (le != cudaSuccess) return sg_cuda_fail(ctx, le, "cudaGraphLaunch");
            SG_CUDA(ctx, cudaMemcpyAsync(ctx->h_scal, s, sizeof(KrylovScalars), cudaMemcpyDeviceToHost, ctx->stream));
            SG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
            ctx->launches += ctx->pcg_per_graph * hs->loops;
        }
        *iters = hs->iters;
        if (!hs->done) return sg_fail(ctx, SGFEM_ERR_MAXIT, "PCG device loop ended before the done flag");
        return hs->status;
    }
};

int status_message(sgfem_context* ctx, int status) {
    if (status == SGFEM_ERR_BREAKDOWN) return sg_fail(ctx, status, "PCG breakdown (p'Ap <= 0 or r'z <= 0)");
    if (status == SGFEM_ERR_NONFINITE) return sg_fail(ctx, status, "non-finite value in a PCG iterate");
    if (status == SGFEM_ERR_MAXIT) return sg_fail(ctx, status, "tolerance not reached within maxit");
    return status;
}

}  // namespace

extern "C" void sgfem_default_options(sgfem_solve_options* o) {
    if (!o) return;
    o->precision = SGFEM_MIXED;
    o->preconditioner = SGFEM_PREC_LATTICE;
    o->rtol = 1e-8;
    o->maxit = 2000;
    o->inner_rtol = 1e-4;  // measured best on the P2 256x256 workload
    o->reference_rhs = 1;
    o->check_every = 4;  // device-loop body length: measured best on the P2 256x256 and sampling workloads
}

extern "C" int sgfem_precondition(sgfem_context* ctx, const double* b, double* y, int kind, int precision) {
    SG_TRY(sg_check_ready(ctx));
    if (!b || !y) return sg_fail(ctx, SGFEM_ERR_ARGUMENT, "null pointer");
    if (precision != SGFEM_FP64 && precision != SGFEM_FP32) return sg_fail(ctx, SGFEM_ERR_ARGUMENT, "bad precision");
    if (kind == SGFEM_PREC_LATTICE && !ctx->lattice)
        return sg_fail(ctx, SGFEM_ERR_UNSUPPORTED, "lattice preconditioner unavailable (dofs do not form a power-of-two lattice)");
    if (kind != SGFEM_PREC_LATTICE && kind != SGFEM_PREC_JACOBI && kind != SGFEM_PREC_NONE && kind != SGFEM_PREC_CHOLESKY)
        return sg_fail(ctx, SGFEM_ERR_ARGUMENT, "bad preconditioner kind");
    SG_CUDA(ctx, cudaSetDevice(ctx->device));
    if (kind == SGFEM_PREC_CHOLESKY) {
        SG_TRY(sg_chol_ensure(ctx));
        SG_TRY(sg_chol_workspace(ctx, SGFEM_FP64));
    }
    const size_t vb = sg_vec_bytes(ctx, precision);
    for (int i = 0; i < 3; ++i) SG_TRY(sg_ensure(ctx, ctx->w_vec[i], vb));
    SG_TRY(sgfem_to_device_layout(ctx, b, ctx->w_vec[0].p, precision));
    SG_CUDA(ctx, cudaMemsetAsync(ctx->w_vec[1].p, 0, vb, ctx->stream));
    if (kind == SGFEM_PREC_LATTICE) {
        SG_TRY(sg_lat_pass_x(ctx, precision, ctx->w_vec[0].p, ctx->w_vec[2].p, nullptr));
        SG_TRY(sg_lat_pass_y(ctx, precision, ctx->w_vec[2].p, nullptr, nullptr, nullptr));
        SG_TRY(sg_lat_pass_xinv(ctx, precision, ctx->w_vec[2].p, ctx->w_vec[1].p, 0, nullptr));
    } else if (kind == SGFEM_PREC_CHOLESKY) {
        SG_TRY(sg_chol_apply(ctx, precision, ctx->w_vec[0].p, ctx->w_vec[1].p, nullptr));
    } else if (kind == SGFEM_PREC_JACOBI) {
        SG_TRY(sg_jacobi(ctx, precision, ctx->w_vec[0].p, ctx->w_vec[1].p, 0, 0, nullptr, nullptr, nullptr));
    } else {
        SG_CUDA(ctx, cudaMemcpyAsync(ctx->w_vec[1].p, ctx->w_vec[0].p, vb, cudaMemcpyDeviceToDevice, ctx->stream));
    }
    return sgfem_from_device_layout(ctx, ctx->w_vec[1].p, y, precision);
}

extern "C" int sgfem_time_precondition(sgfem_context* ctx, int precision, int reps, double* ms_per_application) {
    SG_TRY(sg_check_ready(ctx));
    if (reps <= 0 || !ms_per_application) return sg_fail(ctx, SGFEM_ERR_ARGUMENT, "bad reps");
    if (precision != SGFEM_FP64 && precision != SGFEM_FP32) return sg_fail(ctx, SGFEM_ERR_ARGUMENT, "bad precision");
    SG_CUDA(ctx, cudaSetDevice(ctx->device));
    if (!ctx->lattice) {
        SG_TRY(sg_chol_ensure(ctx));
        SG_TRY(sg_chol_workspace(ctx, SGFEM_FP64));
    }
    const size_t vb = sg_vec_bytes(ctx, precision);
    for (int i = 0; i < 3; ++i) SG_TRY(sg_ensure(ctx, ctx->w_vec[i], vb));
    SG_CUDA(ctx, cudaMemsetAsync(ctx->w_vec[0].p, 0, vb, ctx->stream));
    auto once = [&]() -> int {
        if (!ctx->lattice) return sg_chol_apply(ctx, precision, ctx->w_vec[0].p, ctx->w_vec[1].p, nullptr);
        SG_TRY(sg_lat_pass_x(ctx, precision, ctx->w_vec[0].p, ctx->w_vec[2].p, nullptr));
        SG_TRY(sg_lat_pass_y(ctx, precision, ctx->w_vec[2].p, nullptr, nullptr, nullptr));
        return sg_lat_pass_xinv(ctx, precision, ctx->w_vec[2].p, ctx->w_vec[1].p, 0, nullptr);
    };
    SG_TRY(once());
    SG_CUDA(ctx, cudaEventRecord(ctx->ev0, ctx->stream));
    for (int r = 0; r < reps; ++r) SG_TRY(once());
    SG_CUDA(ctx, cudaEventRecord(ctx->ev1, ctx->stream));
    SG_CUDA(ctx, cudaEventSynchronize(ctx->ev1));
    float ms = 0.f;
    SG_CUDA(ctx, cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
    *ms_per_application = ms / reps;
    return SGFEM_OK;
}

// core solve on device buffers: x64 (in/out, device layout), b0 host (caller order)
// rhs_mode 0: b = (x0 or 0) + e_1 (x) b0 (solve_primal!); 1: b0 in every column (sample problems)
static int solve_core(sgfem_context* ctx, const double* b0, double* x64, const sgfem_solve_options* o,
                      sgfem_solve_stats* st, int rhs_mode) {
    if (o->precision != SGFEM_FP64 && o->precision != SGFEM_FP32 && o->precision != SGFEM_MIXED)
        return sg_fail(ctx, SGFEM_ERR_ARGUMENT, "bad precision");
    int prec_kind = o->preconditioner;
    if (prec_kind == SGFEM_PREC_LATTICE && !ctx->lattice)
        return sg_fail(ctx, SGFEM_ERR_UNSUPPORTED, "lattice preconditioner unavailable (dofs do not form a power-of-two lattice)");
    if (prec_kind != SGFEM_PREC_LATTICE && prec_kind != SGFEM_PREC_JACOBI && prec_kind != SGFEM_PREC_NONE &&
        prec_kind != SGFEM_PREC_CHOLESKY)
        return sg_fail(ctx, SGFEM_ERR_ARGUMENT, "bad preconditioner kind");
    if (!(o->rtol > 0.0) || o->maxit <= 0) return sg_fail(ctx, SGFEM_ERR_ARGUMENT, "rtol must be > 0 and maxit > 0");
    if (prec_kind == SGFEM_PREC_CHOLESKY) {  // factor and size its workspace before any capture
        SG_TRY(sg_chol_ensure(ctx));
        SG_TRY(sg_chol_workspace(ctx, SGFEM_FP64));
    }
    const int check_every = std::max(1, std::min(o->check_every, 64));
    const size_t n64 = sg_vec_bytes(ctx, SGFEM_FP64), n32 = sg_vec_bytes(ctx, SGFEM_FP32);
    const size_t total = (size_t)ctx->n * ctx->ld;
    // buffers: 0 b64, 1 r64, 2 t64/p64, 3 q64, 4 tmp64 ; 5 d32, 6 r32, 7 p32, 8 q32, 9 tmp32
    SG_TRY(sg_ensure(ctx, ctx->w_vec[0], n64));
    SG_TRY(sg_ensure(ctx, ctx->w_vec[1], n64));
    SG_TRY(sg_ensure(ctx, ctx->w_vec[2], n64));
    SG_TRY(sg_ensure(ctx, ctx->w_vec[3], n64));
    SG_TRY(sg_ensure(ctx, ctx->w_vec[4], n64));
    const bool low = o->precision != SGFEM_FP64;
    if (low) {
        for (int i = 5; i < 10; ++i) SG_TRY(sg_ensure(ctx, ctx->w_vec[i], n32));
        SG_TRY(sg_jit_ensure(ctx));
    }
    const int maxblocks = std::max<int>(ctx->num_sms * 8, sg_lat_max_blocks(ctx));
    SG_TRY(sg_ensure(ctx, ctx->w_partials, (size_t)(maxblocks + 8) * sizeof(double)));
    double* partials = (double*)ctx->w_partials.p;
    double* b = (double*)ctx->w_vec[0].p;
    double* r = (double*)ctx->w_vec[1].p;
    double* t = (double*)ctx->w_vec[2].p;
    double* q = (double*)ctx->w_vec[3].p;
    double* tmp = (double*)ctx->w_vec[4].p;

    // b0 upload (caller order) into the staging buffer
    SG_TRY(sg_ensure(ctx, ctx->w_stage, (size_t)ctx->n * sizeof(double) * 2));
    double* d_b0 = (double*)ctx->w_stage.p;
    SG_CUDA(ctx, cudaMemcpyAsync(d_b0, b0, (size_t)ctx->n * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));

    SG_CUDA(ctx, cudaEventRecord(ctx->ev0, ctx->stream));
    const long long launches0 = ctx->launches;
    const int g = vgrid(ctx);
    if (rhs_mode == 1) {
        k_build_rhs_all<<<g, VT, 0, ctx->stream>>>(d_b0, b, ctx->d_iperm, ctx->d_bmask, (int)ctx->n, (int)ctx->P,
                                                  (int)ctx->ld);
        SG_LAUNCHED(ctx);
    } else {
        k_build_rhs<<<g, VT, 0, ctx->stream>>>(d_b0, x64, b, ctx->d_iperm, ctx->d_bmask, (int)ctx->n, (int)ctx->ld,
                                              o->reference_rhs ? 1 : 0);
        ctx->launches++;
        k_add_b0<<<(int)std::min<int64_t>((ctx->n + VT - 1) / VT, 4096), VT, 0, ctx->stream>>>(
            d_b0, b, ctx->d_iperm, ctx->d_bmask, (int)ctx->n, (int)ctx->ld, (int)ctx->imode[0]);
        SG_LAUNCHED(ctx);
    }

    Solver S{ctx, prec_kind, partials, ctx->d_scal};
    // ||b||^2 and ||x0||^2 -> host in one copy (a zero warm start needs no FP64 apply)
    k_dot<double><<<g, VT, 0, ctx->stream>>>(b, b, total, partials);
    double* d_sum = partials + maxblocks + 2;
    SG_TRY(S.fin(g, FIN_SUM, FinArgs{0.0, 0}, d_sum));
    k_dot<double><<<g, VT, 0, ctx->stream>>>(x64, x64, total, partials);
    SG_LAUNCHED(ctx);
    SG_TRY(S.fin(g, FIN_SUM, FinArgs{0.0, 0}, d_sum + 1));
    double bbxx[2] = {0.0, 0.0};
    SG_CUDA(ctx, cudaMemcpyAsync(bbxx, d_sum, 2 * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    SG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    const double bb = bbxx[0], xx = bbxx[1];
    st->iterations = 0;
    st->outer_iterations = 0;
    st->fp64_applies = 0;
    st->relres = 0.0;
    st->apply_ms = -1.0;
    st->precond_ms = -1.0;
    st->kernel_launches = 0;
    if (!std::isfinite(bb)) return sg_fail(ctx, SGFEM_ERR_NONFINITE, "non-finite right-hand side");
    if (bb == 0.0) {
        SG_CUDA(ctx, cudaMemsetAsync(x64, 0, n64, ctx->stream));
        SG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        st->time_ms = 0.0;
        return SGFEM_OK;
    }
    const double rtol2 = o->rtol * o->rtol;

    // true FP64 residual r = b - A x ; returns ||r||^2 on host
    auto true_residual = [&](double* rr_out) -> int {
        int nb = 0;
        SG_TRY(sg_launch_apply(ctx, SGFEM_FP64, x64, t, nullptr, &nb, nullptr));
        k_residual<<<g, VT, 0, ctx->stream>>>(b, t, r, total, partials);
        SG_LAUNCHED(ctx);
        SG_TRY(S.fin(g, FIN_SUM, FinArgs{0.0, 0}, d_sum));
        SG_CUDA(ctx, cudaMemcpyAsync(rr_out, d_sum, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
        SG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        st->fp64_applies += 1;
        return SGFEM_OK;
    };

    // the solution to the caller's pinned host buffer, overlapped with the convergence
    // check that follows: converted on the main stream (one pass over x), copied on the
    // side stream; the host waits for it when the solve returns (sgfem_solve)
    auto spec_out = [&]() -> int {
        if (!ctx->spec_host) return SGFEM_OK;
        if (ctx->spec_pending) SG_CUDA(ctx, cudaStreamWaitEvent(ctx->stream, ctx->ev_spec, 0));  // staging free
        SG_TRY(sg_launch_from_device(ctx, x64, (double*)ctx->w_stage.p, SGFEM_FP64));
        SG_CUDA(ctx, cudaEventRecord(ctx->ev_spec_x, ctx->stream));
        SG_CUDA(ctx, cudaStreamWaitEvent(ctx->side, ctx->ev_spec_x, 0));
        SG_CUDA(ctx, cudaMemcpyAsync(ctx->spec_host, ctx->w_stage.p, (size_t)ctx->n * ctx->P * sizeof(double),
                                     cudaMemcpyDeviceToHost, ctx->side));
        SG_CUDA(ctx, cudaEventRecord(ctx->ev_spec, ctx->side));
        ctx->spec_pending = true;
        ctx->spec_valid = true;
        return SGFEM_OK;
    };

    int status = SGFEM_OK;
    double rr = 0.0;
    // refinement residuals in double-FP32 arithmetic (residual_df.cu) when the operator
    // allows the difference form: x and b as (hi, lo) float pairs, r straight to FP32
    const bool df = low && sg_residual_df_usable(ctx);
    void* xs = nullptr;
    void* bs = nullptr;
    bool r32_ready = false;
    float* r32 = low ? (float*)ctx->w_vec[6].p : nullptr;
    auto residual_df = [&](double* rr_out) -> int {
        int nb = 0;
        SG_TRY(sg_residual_df(ctx, xs, bs, r32, partials, &nb));
        SG_TRY(S.fin(nb, FIN_SUM, FinArgs{0.0, 0}, d_sum));
        SG_CUDA(ctx, cudaMemcpyAsync(rr_out, d_sum, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
        SG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        r32_ready = true;
        return SGFEM_OK;
    };
    if (df) {
        SG_TRY(sg_residual_df_prepare(ctx));
        SG_TRY(sg_ensure(ctx, ctx->w_vec[12], n64));
        SG_TRY(sg_ensure(ctx, ctx->w_vec[13], n64));
        xs = ctx->w_vec[12].p;
        bs = ctx->w_vec[13].p;
        SG_TRY(sg_split_df(ctx, b, nullptr, bs, 0));
    }
    {
        // initial residual: with a zero warm start r = b and no FP64 apply is needed
        if (xx == 0.0) {
            SG_CUDA(ctx, cudaMemcpyAsync(r, b, n64, cudaMemcpyDeviceToDevice, ctx->stream));
            rr = bb;
        } else if (df) {
            SG_TRY(sg_split_df(ctx, x64, nullptr, xs, 0));
            SG_TRY(residual_df(&rr));
        } else {
            SG_TRY(true_residual(&rr));
        }
    }
    int remaining = o->maxit;
    // SGFEM_TRACE=1: one line per refinement step on stderr (the reference's @info progress)
    const char* etr = getenv("SGFEM_TRACE");
    const int trace = etr ? atoi(etr) : 0;  // 2: also the recurrence and FP32-operator residuals
    // smallest reduction asked of one later refinement step (SGFEM_MIXED_FLOOR)
    const char* efl = getenv("SGFEM_MIXED_FLOOR");
    const double floor1 = efl ? std::max(1e-10, std::min(1e-2, atof(efl))) : 1e-6;
    const double floor2 = floor1 * floor1;
    // sample problems: the global residual is driven down until every column
    // meets rtol relative to its own right-hand side
    double tol2e = rtol2;
    double colmax = 0.0;
    std::vector<double> cr, cb;
    for (int pass = 0; pass < 6; ++pass) {
        if (!low) {
            // FP64 PCG; restart from the true residual if the recurrence drifted
            for (int restart = 0; restart < 8; ++restart) {
                if (!std::isfinite(rr)) { status = SGFEM_ERR_NONFINITE; break; }
                if (rr <= tol2e * bb || remaining <= 0) break;
                KrylovScalars h{};
                h.tol2 = tol2e * bb;
                SG_CUDA(ctx, cudaMemcpyAsync(ctx->d_scal, &h, sizeof(KrylovScalars), cudaMemcpyHostToDevice, ctx->stream));
                int it = 0;
                ctx->spec_valid = false;
                status = S.pcg<double>(SGFEM_FP64, x64, r, t, q, tmp, remaining, check_every, &it);
                st->iterations += it;
                st->outer_iterations += 1;
                remaining -= it;
                if (status == SGFEM_OK) SG_TRY(spec_out());  // the recurrence met the target
                SG_TRY(true_residual(&rr));
                if (status != SGFEM_OK) break;
            }
        } else {
            float* d32 = (float*)ctx->w_vec[5].p;
            double* d64 = q;  // the FP32 PCG's solution, accumulated in FP64
            float* p32 = (float*)ctx->w_vec[7].p;
            float* q32 = (float*)ctx->w_vec[8].p;
            float* tmp32 = (float*)ctx->w_vec[9].p;
            const double in2 = o->precision == SGFEM_FP32 ? tol2e : o->inner_rtol * o->inner_rtol;
            // small P1 lattice problems: the inner FP32 PCG in one cluster launch (SGFEM_SMALL=0 disables)
            const bool use_small = prec_kind == SGFEM_PREC_LATTICE && !ctx->batched && sg_small_usable(ctx);
            for (int outer = 0; outer < 64; ++outer) {
                if (!std::isfinite(rr)) { status = SGFEM_ERR_NONFINITE; break; }
                if (rr <= tol2e * bb) break;
                if (remaining <= 0) { status = SGFEM_ERR_MAXIT; break; }
                if (r32_ready) {  // the double-FP32 residual already wrote the FP32 right-hand side
                    SG_CUDA(ctx, cudaMemsetAsync(d64, 0, n64, ctx->stream));
                    k_dot<float><<<g, VT, 0, ctx->stream>>>(r32, r32, total, partials);  // for FIN_TOL below
                    SG_LAUNCHED(ctx);
                    if (trace >= 2) {  // the diagnostics compare against r in FP64
                        k_to_f64<<<g, VT, 0, ctx->stream>>>(r32, r, total);
                        SG_LAUNCHED(ctx);
                    }
                } else {
                    k_demote<<<g, VT, 0, ctx->stream>>>(r, r32, d64, total, partials);
                    SG_LAUNCHED(ctx);
                }
                // inner target (squared reduction of ||r||).  First step: inner_rtol.  Later
                // steps aim to end the solve with a margin of 3, asking at most a 1e-6
                // reduction of one FP32 PCG (about what its recurrence tracks in FP64 with
                // the solution accumulated in FP64; SGFEM_TRACE=2 prints both per step).
                const double finish = 0.1 * tol2e * bb / rr;
                double want;
                if (o->precision == SGFEM_FP32) want = std::max(in2, 0.25 * tol2e * bb / rr);
                else if (outer == 0) want = std::max(in2, finish);
                else want = std::max(finish, floor2);
                SG_TRY(S.fin(g, FIN_TOL, FinArgs{want, 0}, nullptr));
                int it = 0;
                int s2 = SGFEM_OK;
                if (use_small) {  // the whole FP32 PCG in one cluster launch (small.cu), no host wait:
                    // iterations and status are read with the refinement residual below
                    SG_CUDA(ctx, cudaMemsetAsync(d64, 0, n64, ctx->stream));
                    SG_TRY(sg_small_pcg_launch(ctx, r32, d64, remaining));
                } else {
                    s2 = S.pcg<float, double>(SGFEM_FP32, d64, r32, p32, q32, tmp32, remaining, check_every, &it);
                    st->iterations += it;
                    st->outer_iterations += 1;
                    remaining -= it;
                    if (s2 == SGFEM_ERR_BREAKDOWN || s2 == SGFEM_ERR_NONFINITE) { status = s2; break; }
                }
                double rec = 0.0, tr32 = 0.0;
                if (trace >= 2) {  // recurrence ||r32|| and FP32-operator residual ||r - A32 d|| (one extra apply)
                    k_dot<float><<<g, VT, 0, ctx->stream>>>(r32, r32, total, partials);
                    SG_LAUNCHED(ctx);
                    SG_TRY(S.fin(g, FIN_SUM, FinArgs{0.0, 0}, d_sum));
                    SG_CUDA(ctx, cudaMemcpyAsync(&rec, d_sum, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
                    k_to_f32<<<g, VT, 0, ctx->stream>>>(d64, d32, total);
                    SG_LAUNCHED(ctx);
                    SG_TRY(sg_launch_apply(ctx, SGFEM_FP32, d32, q32, nullptr, nullptr, nullptr));
                    k_diffnorm<<<g, VT, 0, ctx->stream>>>(r, q32, total, partials);
                    SG_LAUNCHED(ctx);
                    SG_TRY(S.fin(g, FIN_SUM, FinArgs{0.0, 0}, d_sum));
                    SG_CUDA(ctx, cudaMemcpyAsync(&tr32, d_sum, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
                    SG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
                }
                const double rr_in = rr;
                // a step whose target reduction reaches the final tolerance (or the single FP32
                // solve) is expected to end the solve
                const bool last = o->precision == SGFEM_FP32 || rr * want <= tol2e * bb;
                ctx->spec_valid = false;
                if (df) {
                    SG_TRY(sg_split_df(ctx, x64, d64, xs, 1));  // x += d, then x as (hi, lo)
                    if (last) SG_TRY(spec_out());
                    SG_TRY(residual_df(&rr));
                } else {
                    k_add64<<<g, VT, 0, ctx->stream>>>(x64, d64, total);
                    SG_LAUNCHED(ctx);
                    if (last) SG_TRY(spec_out());
                    SG_TRY(true_residual(&rr));
                }
                if (use_small) {  // the residual's synchronisation also brought the scalars
                    sg_small_pcg_result(ctx, &it, &s2);
                    if (s2 == SGFEM_ERR_MAXIT) s2 = SGFEM_OK;  // the outer loop reports it
                    st->iterations += it;
                    st->outer_iterations += 1;
                    remaining -= it;
                    // a failed inner solve returned d = 0: x and r are the previous step's
                    if (s2 == SGFEM_ERR_BREAKDOWN || s2 == SGFEM_ERR_NONFINITE) { status = s2; break; }
                }
                if (trace)
                    fprintf(stderr, "sgfem: refinement step %d: inner target %.3g, %d FP32 iterations, relres %.3e\n",
                            outer + 1, std::sqrt(want), it, std::sqrt(rr / bb));
                if (trace >= 2)
                    fprintf(stderr, "sgfem:   reduction: recurrence %.3e, FP32 operator %.3e, %s %.3e\n",
                            std::sqrt(rec / rr_in), std::sqrt(tr32 / rr_in), df ? "double-FP32" : "FP64",
                            std::sqrt(rr / rr_in));
                if (o->precision == SGFEM_FP32) break;  // plain FP32 PCG: no refinement
            }
        }
        if (!ctx->batched || status != SGFEM_OK) break;
        const int S = (int)ctx->P;
        cr.resize(S);
        cb.resize(S);
        double* d_cols = partials;  // S column norms (partials is no longer in use)
        k_colnorm2<<<S, VT, 0, ctx->stream>>>(r, (int)ctx->n, (int)ctx->ld, d_cols);
        SG_LAUNCHED(ctx);
        SG_CUDA(ctx, cudaMemcpyAsync(cr.data(), d_cols, S * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
        k_colnorm2<<<S, VT, 0, ctx->stream>>>(b, (int)ctx->n, (int)ctx->ld, d_cols);
        SG_LAUNCHED(ctx);
        SG_CUDA(ctx, cudaMemcpyAsync(cb.data(), d_cols, S * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
        SG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        colmax = 0.0;
        for (int c = 0; c < S; ++c)
            if (cb[c] > 0.0) colmax = std::max(colmax, std::sqrt(cr[c] / cb[c]));
        if (colmax <= o->rtol) break;
        tol2e = std::min(tol2e, rr / bb) * 0.25 * (o->rtol / colmax) * (o->rtol / colmax);
    }
    SG_CUDA(ctx, cudaEventRecord(ctx->ev1, ctx->stream));
    SG_CUDA(ctx, cudaEventSynchronize(ctx->ev1));
    float ms = 0.f;
    SG_CUDA(ctx, cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
    st->time_ms = ms;
    st->kernel_launches = ctx->launches - launches0;
    if (low) SG_TRY(sg_jit_check(ctx));
    st->relres = ctx->batched ? colmax : std::sqrt(rr / bb);
    if (status == SGFEM_OK && !(st->relres <= o->rtol)) status = (o->precision == SGFEM_FP32) ? SGFEM_OK : SGFEM_ERR_MAXIT;
    return status_message(ctx, status);
}

extern "C" int sgfem_solve_device(sgfem_context* ctx, const double* b0, void* x_dev, const sgfem_solve_options* opts,
                                  sgfem_solve_stats* stats) {
    SG_TRY(sg_check_ready(ctx));
    if (!b0 || !x_dev) return sg_fail(ctx, SGFEM_ERR_ARGUMENT, "null pointer");
    sgfem_solve_options o;
    if (opts) o = *opts; else sgfem_default_options(&o);
    sgfem_solve_stats s{};
    SG_CUDA(ctx, cudaSetDevice(ctx->device));
    int rc = solve_core(ctx, b0, (double*)x_dev, &o, &s, 0);
    if (stats) *stats = s;
    return rc;
}

extern "C" int sgfem_solve(sgfem_context* ctx, const double* b0, double* x_inout, const sgfem_solve_options* opts,
                           sgfem_solve_stats* stats) {
    SG_TRY(sg_check_ready(ctx));
    if (!b0 || !x_inout) return sg_fail(ctx, SGFEM_ERR_ARGUMENT, "null pointer");
    SG_CUDA(ctx, cudaSetDevice(ctx->device));
    const size_t n64 = sg_vec_bytes(ctx, SGFEM_FP64);
    SG_TRY(sg_ensure(ctx, ctx->w_vec[10], n64));
    ctx->samples_x_valid = false;
    SG_TRY(sgfem_to_device_layout(ctx, x_inout, ctx->w_vec[10].p, SGFEM_FP64));
    // pinned x_inout: the solution's copy overlaps the last convergence check
    // (SGFEM_OVERLAP_COPY=0 turns this off); pageable memory takes the copy below
    cudaPointerAttributes pa{};
    const bool pinned = cudaPointerGetAttributes(&pa, x_inout) == cudaSuccess && pa.type == cudaMemoryTypeHost;
    cudaGetLastError();
    const char* eov = getenv("SGFEM_OVERLAP_COPY");
    if (pinned && !(eov && atoi(eov) == 0)) {
        if (!ctx->side) SG_CUDA(ctx, cudaStreamCreateWithFlags(&ctx->side, cudaStreamNonBlocking));
        if (!ctx->ev_spec_x) SG_CUDA(ctx, cudaEventCreateWithFlags(&ctx->ev_spec_x, cudaEventDisableTiming));
        if (!ctx->ev_spec) SG_CUDA(ctx, cudaEventCreateWithFlags(&ctx->ev_spec, cudaEventDisableTiming));
        ctx->spec_host = x_inout;
    }
    ctx->spec_pending = false;
    ctx->spec_valid = false;
    int rc = sgfem_solve_device(ctx, b0, ctx->w_vec[10].p, opts, stats);
    ctx->spec_host = nullptr;
    if (ctx->spec_pending) {  // a copy into x_inout may still run: wait for it on every return
        ctx->spec_pending = false;
        const cudaError_t e = cudaEventSynchronize(ctx->ev_spec);
        if (e != cudaSuccess) return sg_cuda_fail(ctx, e, "solution copy");
        if (ctx->spec_valid && (rc == SGFEM_OK || rc == SGFEM_ERR_MAXIT)) {
            if (getenv("SGFEM_TRACE")) fprintf(stderr, "sgfem: solution copy overlapped with the convergence check\n");
            return rc;  // x_inout holds the final solution
        }
    }
    if (rc != SGFEM_OK && rc != SGFEM_ERR_MAXIT) return rc;
    std::string keep = ctx->err;
    int rc2 = sgfem_from_device_layout(ctx, ctx->w_vec[10].p, x_inout, SGFEM_FP64);
    if (rc2 != SGFEM_OK) return rc2;
    ctx->err = keep;
    return rc;
}

extern "C" int sgfem_solve_samples(sgfem_context* ctx, const double* b0, double* x_inout,
                                   const sgfem_solve_options* opts, sgfem_solve_stats* stats) {
    SG_TRY(sg_check_ready(ctx));
    if (!ctx->batched) return sg_fail(ctx, SGFEM_ERR_STATE, "sgfem_solve_samples needs a context set up with sgfem_set_samples");
    if (!b0) return sg_fail(ctx, SGFEM_ERR_ARGUMENT, "null pointer");
    sgfem_solve_options o;
    if (opts) o = *opts; else sgfem_default_options(&o);
    SG_CUDA(ctx, cudaSetDevice(ctx->device));
    const size_t n64 = sg_vec_bytes(ctx, SGFEM_FP64);
    SG_TRY(sg_ensure(ctx, ctx->w_vec[10], n64));
    ctx->samples_x_valid = false;
    if (x_inout)
        SG_TRY(sgfem_to_device_layout(ctx, x_inout, ctx->w_vec[10].p, SGFEM_FP64));
    else
        SG_CUDA(ctx, cudaMemsetAsync(ctx->w_vec[10].p, 0, n64, ctx->stream));
    sgfem_solve_stats s{};
    int rc = solve_core(ctx, b0, (double*)ctx->w_vec[10].p, &o, &s, 1);
    if (stats) *stats = s;
    if (rc != SGFEM_OK && rc != SGFEM_ERR_MAXIT) return rc;
    ctx->samples_x_valid = rc == SGFEM_OK;
    if (!x_inout) return rc;
    std::string keep = ctx->err;
    int rc2 = sgfem_from_device_layout(ctx, ctx->w_vec[10].p, x_inout, SGFEM_FP64);
    if (rc2 != SGFEM_OK) return rc2;
    ctx->err = keep;
    return rc;
}
