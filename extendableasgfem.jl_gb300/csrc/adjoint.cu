// K6: contractions of the adjoint gradient of a mean quantity of interest.
//
// No counterpart in the reference package (its Julia API has no derivative).
// For PoissonProblemPrimal the SG system (src/modelproblems/solvers_poisson_primal.jl:86-124)
//   S U = b,   S = I (x) K_0 + sum_m G_m (x) K_m,
// with K_0 = (a_0 grad u, grad v), a_0 = sum_i alpha_i phi_i a nodal P1 mean field, and
// J = l . U_0 (U_0 the mean mode, E[u] for an orthonormal basis), the adjoint
// S^T Lambda = e_1 (x) l gives (S is symmetric, so the same PCG solves it)
//   dJ/dt_m     = -Lambda^T (G_m (x) K_m) U      (t_m multiplies block m, m = 1..M)
//   dJ/dalpha_i = -sum_mu Lambda_mu^T K_0^(i) U_mu,  K_0^(i) = (phi_i grad u, grad v)
//               = -sum_{T containing i} (|T| / 3) sum_mu grad Lambda_mu . grad U_mu   (P1)
// Kernels
//   k_adj_blocks  one warp per matrix row, lanes over the couplings (m, mu, nu, g):
//                 g Lambda[i, mu] sum_j K_m[i, j] U[j, nu], summed per m into lane-private
//                 shared-memory slots, then per-warp partials reduced in a fixed order.
//   k_adj_cells   one warp per cell, lanes over modes: (|T|/3) sum_mu grad Lambda_mu . grad U_mu.
//   k_adj_nodes   one thread per node: minus the sum over its cells in ascending order.
// FP64 throughout; bitwise reproducible.
#include <algorithm>
#include <cmath>
#include <vector>

#include "sgfem_internal.h"

namespace {

struct Coupling {
    int m;      // 1..M
    int cmu;    // device column of mu
    int cnu;    // device column of nu
    double g;
};

__global__ void k_adj_blocks(const int* __restrict__ rowptr, const int* __restrict__ col,
                             const double* __restrict__ vals, int M1, const double* __restrict__ U,
                             const double* __restrict__ Lam, int n, int ld, const Coupling* __restrict__ cp, int E,
                             int wpb, double* __restrict__ partials) {
    extern __shared__ double accm[];  // [warp][M1][32]
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    double* acc = accm + (size_t)warp * M1 * 32;
    for (int m = 0; m < M1; ++m) acc[m * 32 + lane] = 0.0;
    const int nw = gridDim.x * wpb, w = blockIdx.x * wpb + warp;
    for (int i = w; i < n; i += nw) {
        const int a = rowptr[i], b = rowptr[i + 1];
        for (int e0 = 0; e0 < E; e0 += 32) {
            const int e = e0 + lane;
            Coupling c{0, 0, 0, 0.0};
            if (e < E) c = cp[e];
            const double lg = (e < E) ? c.g * Lam[(size_t)i * ld + c.cmu] : 0.0;
            double s = 0.0;
            for (int k = a; k < b; ++k) {
                const int j = col[k];
                s = fma(vals[(size_t)k * M1 + c.m], U[(size_t)j * ld + c.cnu], s);
            }
            if (e < E) acc[c.m * 32 + lane] = fma(lg, s, acc[c.m * 32 + lane]);
        }
    }
    __syncwarp();
    for (int m = 0; m < M1; ++m) {
        double v = acc[m * 32 + lane];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (lane == 0) partials[(size_t)w * M1 + m] = v;
    }
}

// out[m] = -sum_w partials[w * M1 + m], fixed order
__global__ void k_adj_blocks_fin(const double* __restrict__ partials, int nw, int M1, double* __restrict__ out) {
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= M1) return;
    double s = 0.0;
    for (int w = 0; w < nw; ++w) s += partials[(size_t)w * M1 + m];
    out[m] = -s;
}

struct Tri {
    int r[3];      // device rows of the three vertex dofs
    double g[6];   // grad lambda_0..2
    double vol3;   // |T| / 3
};

__global__ void k_adj_cells(const Tri* __restrict__ tri, int nc, const double* __restrict__ U,
                            const double* __restrict__ Lam, int P, int ld, double* __restrict__ cval) {
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    for (int c = warp; c < nc; c += nw) {
        const Tri T = tri[c];
        double s = 0.0;
        for (int k = lane; k < P; k += 32) {
            double lx = 0.0, ly = 0.0, ux = 0.0, uy = 0.0;
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                const double l = Lam[(size_t)T.r[a] * ld + k], u = U[(size_t)T.r[a] * ld + k];
                lx = fma(l, T.g[2 * a], lx);
                ly = fma(l, T.g[2 * a + 1], ly);
                ux = fma(u, T.g[2 * a], ux);
                uy = fma(u, T.g[2 * a + 1], uy);
            }
            s = fma(lx, ux, fma(ly, uy, s));
        }
        for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
        if (lane == 0) cval[c] = s * T.vol3;
    }
}

__global__ void k_adj_nodes(const int* __restrict__ nptr, const int* __restrict__ ncell,
                            const double* __restrict__ cval, int nn, double* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nn) return;
    double s = 0.0;
    for (int k = nptr[i]; k < nptr[i + 1]; ++k) s += cval[ncell[k]];
    out[i] = -s;
}

struct Owned {
    std::vector<void*> p;
    ~Owned() {
        for (void* q : p) cudaFree(q);
    }
};

template <typename T>
int up(sgfem_context* ctx, Owned& o, const T* src, size_t n, T** dst) {
    void* p = nullptr;
    SG_CUDA(ctx, cudaMalloc(&p, std::max<size_t>(n, 1) * sizeof(T)));
    o.p.push_back(p);
    if (n) SG_CUDA(ctx, cudaMemcpyAsync(p, src, n * sizeof(T), cudaMemcpyHostToDevice, ctx->stream));
    *dst = (T*)p;
    return SGFEM_OK;
}

}  // namespace

extern "C" int sgfem_adjoint_gradient(sgfem_context* ctx, const double* U, const double* Lambda, double* dblocks,
                                      const sgfem_mesh* mesh, double* dalpha) {
    SG_TRY(sg_check_ready(ctx));
    if (ctx->batched) return sg_fail(ctx, SGFEM_ERR_STATE, "sgfem_adjoint_gradient: samples context");
    if (!U || !Lambda || (!dblocks && !dalpha) || (dalpha && !mesh))
        return sg_fail(ctx, SGFEM_ERR_ARGUMENT, "sgfem_adjoint_gradient: null argument");
    SG_CUDA(ctx, cudaSetDevice(ctx->device));
    const int64_t n = ctx->n, P = ctx->P, M = ctx->M;
    const int M1 = ctx->M1, ld = (int)ctx->ld;
    const size_t n64 = sg_vec_bytes(ctx, SGFEM_FP64);
    SG_TRY(sg_ensure(ctx, ctx->w_vec[0], n64));
    SG_TRY(sg_ensure(ctx, ctx->w_vec[1], n64));
    SG_TRY(sgfem_to_device_layout(ctx, U, ctx->w_vec[0].p, SGFEM_FP64));
    SG_TRY(sgfem_to_device_layout(ctx, Lambda, ctx->w_vec[1].p, SGFEM_FP64));
    const double* dU = (const double*)ctx->w_vec[0].p;
    const double* dL = (const double*)ctx->w_vec[1].p;
    Owned o;

    if (dblocks) {
        std::vector<Coupling> cps;
        for (int64_t nu = 0; nu < P; ++nu)
            for (int64_t k = ctx->G_colptr[nu]; k < ctx->G_colptr[nu + 1]; ++k) {
                const double g = ctx->G_val[k];
                if (g == 0.0) continue;
                const int64_t r = ctx->G_rowval[k];
                cps.push_back({(int)(r / P) + 1, ctx->imode[r % P], ctx->imode[nu], g});
            }
        std::stable_sort(cps.begin(), cps.end(), [](const Coupling& x, const Coupling& y) { return x.m < y.m; });
        const int E = (int)cps.size();
        if (M > 0) {
            int wpb = 4;
            while (wpb > 1 && (size_t)wpb * M1 * 32 * sizeof(double) > 200 * 1024) --wpb;
            const size_t smem = (size_t)wpb * M1 * 32 * sizeof(double);
            if (smem > 200 * 1024) return sg_fail(ctx, SGFEM_ERR_UNSUPPORTED, "too many KLE terms for the gradient kernel");
            const int blocks = std::max(1, std::min<int>((int)((n + wpb - 1) / wpb), ctx->num_sms * 8));
            const int nw = blocks * wpb;
            Coupling* d_cp;
            double *d_part, *d_out;
            SG_TRY(up(ctx, o, cps.data(), cps.size(), &d_cp));
            SG_CUDA(ctx, cudaMalloc((void**)&d_part, (size_t)nw * M1 * sizeof(double)));
            o.p.push_back(d_part);
            SG_CUDA(ctx, cudaMalloc((void**)&d_out, (size_t)M1 * sizeof(double)));
            o.p.push_back(d_out);
            if (smem > 48 * 1024)
                SG_CUDA(ctx, cudaFuncSetAttribute(k_adj_blocks, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
            k_adj_blocks<<<blocks, wpb * 32, smem, ctx->stream>>>(ctx->d_rowptr, ctx->d_col, ctx->d_val64, M1, dU, dL,
                                                                (int)n, ld, d_cp, E, wpb, d_part);
            SG_LAUNCHED(ctx);
            k_adj_blocks_fin<<<(M1 + 127) / 128, 128, 0, ctx->stream>>>(d_part, nw, M1, d_out);
            SG_LAUNCHED(ctx);
            std::vector<double> out(M1);
            SG_CUDA(ctx, cudaMemcpyAsync(out.data(), d_out, M1 * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
            SG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
            for (int64_t m = 1; m <= M; ++m) dblocks[m - 1] = out[m];
        }
    }

    if (dalpha) {
        if (mesh->order != 1) return sg_fail(ctx, SGFEM_ERR_UNSUPPORTED, "mean-field gradient needs the P1 space");
        const int64_t nc = mesh->ncells, nn = mesh->nnodes;
        if (nc <= 0 || nn != n || !mesh->coords || !mesh->cell_nodes || !mesh->cell_volumes)
            return sg_fail(ctx, SGFEM_ERR_ARGUMENT, "mesh: P1 space with one dof per node expected");
        std::vector<Tri> tri(nc);
        std::vector<int> cnt(nn + 1, 0);
        for (int64_t c = 0; c < nc; ++c) {
            const int64_t* cn = mesh->cell_nodes + 3 * c;
            double px[3], py[3];
            for (int k = 0; k < 3; ++k) {
                const int64_t v = cn[k] - 1;
                if (v < 0 || v >= nn) return sg_fail(ctx, SGFEM_ERR_ARGUMENT, "cell_nodes out of range");
                px[k] = mesh->coords[2 * v];
                py[k] = mesh->coords[2 * v + 1];
                tri[c].r[k] = ctx->iperm[v];
                cnt[v + 1]++;
            }
            const double j00 = px[1] - px[0], j01 = px[2] - px[0], j10 = py[1] - py[0], j11 = py[2] - py[0];
            const double det = j00 * j11 - j01 * j10;
            if (det == 0.0) return sg_fail(ctx, SGFEM_ERR_ARGUMENT, "degenerate cell");
            const double i00 = j11 / det, i01 = -j01 / det, i10 = -j10 / det, i11 = j00 / det;
            Tri& T = tri[c];
            T.g[2] = i00; T.g[3] = i01;
            T.g[4] = i10; T.g[5] = i11;
            T.g[0] = -i00 - i10; T.g[1] = -i01 - i11;
            T.vol3 = mesh->cell_volumes[c] / 3.0;
        }
        for (int64_t i = 0; i < nn; ++i) cnt[i + 1] += cnt[i];
        std::vector<int> ncell(cnt[nn]);
        std::vector<int> fill(cnt.begin(), cnt.end() - 1);
        for (int64_t c = 0; c < nc; ++c)
            for (int k = 0; k < 3; ++k) ncell[fill[mesh->cell_nodes[3 * c + k] - 1]++] = (int)c;
        Tri* d_tri;
        int *d_nptr, *d_ncell;
        double *d_cval, *d_out;
        SG_TRY(up(ctx, o, tri.data(), tri.size(), &d_tri));
        SG_TRY(up(ctx, o, cnt.data(), cnt.size(), &d_nptr));
        SG_TRY(up(ctx, o, ncell.data(), ncell.size(), &d_ncell));
        SG_CUDA(ctx, cudaMalloc((void**)&d_cval, (size_t)nc * sizeof(double)));
        o.p.push_back(d_cval);
        SG_CUDA(ctx, cudaMalloc((void**)&d_out, (size_t)nn * sizeof(double)));
        o.p.push_back(d_out);
        const int blocks = (int)std::min<int64_t>((nc + 7) / 8, (int64_t)ctx->num_sms * 16);
        k_adj_cells<<<blocks, 256, 0, ctx->stream>>>(d_tri, (int)nc, dU, dL, (int)P, ld, d_cval);
        SG_LAUNCHED(ctx);
        k_adj_nodes<<<(int)((nn + 255) / 256), 256, 0, ctx->stream>>>(d_nptr, d_ncell, d_cval, (int)nn, d_out);
        SG_LAUNCHED(ctx);
        SG_CUDA(ctx, cudaMemcpyAsync(dalpha, d_out, (size_t)nn * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
        SG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    }
    return SGFEM_OK;
}
