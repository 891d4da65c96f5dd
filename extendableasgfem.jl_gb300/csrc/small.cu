// The FP32 inner PCG of the mixed solve for small problems in ONE launch: a
// thread-block cluster keeps the SG vectors in its shared memory (distributed
// shared memory between its CTAs) and runs every iteration (operator apply,
// exact mean-based preconditioner, dot products, updates) with cluster barriers
// between the phases instead of kernel launches.  The iterates are those of the
// multi-launch FP32 PCG (krylov.cu) on the same system: the reference's
// mul! (src/modelproblems/solvers_poisson_primal.jl:86-124) and ldiv! with
// LU(K_0) (:47-78), here for K_0 = a0 * (5-point Laplacian) on the interior
// points of a power-of-two dof lattice (P1 on the unit square with a constant
// mean, config 1), whose inverse is the 2-D sine transform
//   K_0^-1 = S diag(1 / (a0 (lam_kx + lam_ky))) S,  S_kx = sqrt(2/Nl) sin(pi k x / Nl),
//   lam_k = 4 sin^2(pi k / (2 Nl)).
// Small problems spend their time in launch and synchronisation latency (a
// config-1 iteration is ~8 launches of a few microseconds each); one cluster
// launch per refinement step removes that.
//
// Layout: CTA b of the cluster owns the lattice lines [lo(b), lo(b+1)) (all
// modes; lane = device column, ld <= 32), its rows of r, p, q, z in shared
// memory.  Apply: a warp per row, the X rows of neighbouring lines read from the
// owning CTA's shared memory; per row w_m = sum_j K_m[i,j] (p_j - p_i)
// (difference form) for every KLE term, then q_mu = w_0[mu] + sum g w_m[nu] with
// nu fetched by warp shuffles from the lane that owns it.  Preconditioner:
// x-transform of the CTA's lines, then CTA b transforms the columns kx of its
// share along y (scale, back along y), then the x-transform back of its lines;
// the two changes of ownership read the other CTAs' shared memory.  Dot
// products: per-CTA FP64 partials, summed by every CTA in rank order (all CTAs
// take identical decisions).  The FP64 solution correction accumulates in
// global memory (x += alpha p in FP64, as in the multi-launch solve).
#include <cooperative_groups.h>

#include <cmath>
#include <string>
#include <vector>

#include "sgfem_internal.h"

namespace cg = cooperative_groups;

namespace {

constexpr int SM_THREADS = 512;
constexpr int SM_WARPS = SM_THREADS / 32;
constexpr int SM_MAXM1 = 16;   // KLE terms (M + 1) the kernel holds per row
constexpr int SM_MAXSLOT = 4;  // couplings per (term, output mode)

struct SmallGeom {
    int NP;      // lattice points per line (Nl + 1)
    int N;       // interior points per line (Nl - 1)
    int NS;      // row stride of the sine matrix (N rounded up to 4)
    int ld, M1, M1P;
    int CL;      // CTAs in the cluster
    int MAXL;    // lines per CTA (most)
    int MAXK;    // transform columns per CTA (most)
    int diff;
};

struct SmallTabs {
    const float* S;       // N x NS, S[k][x] (symmetric)
    const float* scale;   // N x N, 1 / (a0 (lam_ky + lam_kx)), [ky][kx]
    const int* nslot;     // [M1]: couplings per output mode for term m (max over modes)
    const int* src;       // [M1][SM_MAXSLOT][32]: source lane (device column)
    const float* g;       // [M1][SM_MAXSLOT][32]: coefficient (0 for padding)
};

__device__ __forceinline__ int line_lo(int b, const SmallGeom& G) { return (int)(((long long)b * G.NP) / G.CL); }
__device__ __forceinline__ int col_lo(int b, const SmallGeom& G) { return (int)(((long long)b * G.N) / G.CL); }

__global__ void __launch_bounds__(SM_THREADS, 1)
k_small_pcg(const int* __restrict__ rowptr, const int* __restrict__ col, const float* __restrict__ vals,
            const unsigned char* __restrict__ bmask, const float* __restrict__ rin, double* __restrict__ x64,
            KrylovScalars* __restrict__ scal, SmallTabs tb, SmallGeom G, int maxit) {
    cg::cluster_group cluster = cg::this_cluster();
    const int me = (int)cluster.block_rank();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    extern __shared__ __align__(16) float sm[];
    const int RMAX = G.MAXL * G.NP;
    float* r_s = sm;
    float* p_s = r_s + RMAX * 32;
    float* q_s = p_s + RMAX * 32;
    float* z_s = q_s + RMAX * 32;
    float* T_s = z_s + RMAX * 32;                 // [MAXL][N][32]: x-transform of my lines
    float* Tl_s = T_s + G.MAXL * G.N * 32;        // [N][MAXK][32]: my columns, all lines
    float* V_s = Tl_s + G.N * G.MAXK * 32;        // [N][MAXK][32]: my columns after y, scale, y
    float* Vl_s = V_s + G.N * G.MAXK * 32;        // [MAXL][N][32]: all columns of my lines
    float* S_s = Vl_s + G.MAXL * G.N * 32;        // [N][NS]
    int* owner_s = reinterpret_cast<int*>(S_s + G.N * G.NS);  // [NP]
    int* src_s = owner_s + ((G.NP + 3) & ~3);                   // [M1][SM_MAXSLOT][32]
    float* g_s = reinterpret_cast<float*>(src_s + G.M1 * SM_MAXSLOT * 32);
    double* red_s = reinterpret_cast<double*>(g_s + ((G.M1 * SM_MAXSLOT * 32 + 1) & ~1));  // [3]: pq, rr, rz
    __shared__ double wred[SM_WARPS];
    __shared__ int nslot_s[SM_MAXM1];

    const int l0 = line_lo(me, G), l1 = line_lo(me + 1, G);
    const int nrow = (l1 - l0) * G.NP;
    const int row0 = l0 * G.NP;
    const int k0 = col_lo(me, G), k1 = col_lo(me + 1, G);
    const int nk = k1 - k0;
    const bool lv = lane < G.ld;
    for (int i = threadIdx.x; i < G.N * G.NS; i += SM_THREADS) S_s[i] = tb.S[i];
    for (int y = threadIdx.x; y < G.NP; y += SM_THREADS) {
        int o = 0;
        while (o + 1 < G.CL && line_lo(o + 1, G) <= y) ++o;
        owner_s[y] = o;
    }
    for (int i = threadIdx.x; i < RMAX * 32; i += SM_THREADS) {
        const int li = i >> 5, c = i & 31;
        const float v = (li < nrow && c < G.ld) ? rin[(size_t)(row0 + li) * G.ld + c] : 0.f;
        r_s[i] = v;
        p_s[i] = 0.f;
        q_s[i] = 0.f;
        z_s[i] = 0.f;
    }
    // coupling tables of the apply (per term m, slot s and output lane: source lane, g)
    for (int i = threadIdx.x; i < G.M1 * SM_MAXSLOT * 32; i += SM_THREADS) {
        src_s[i] = tb.src[i];
        g_s[i] = tb.g[i];
    }
    if (threadIdx.x < SM_MAXM1) nslot_s[threadIdx.x] = threadIdx.x < G.M1 ? tb.nslot[threadIdx.x] : 0;
    __syncthreads();
    const double tol2 = scal->tol2;

    // cluster-wide sum of one FP64 value per thread: warp, then CTA, then the CTAs in rank order
    auto csum = [&](double v, int slot) -> double {
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (lane == 0) wred[warp] = v;
        __syncthreads();
        if (threadIdx.x == 0) {
            double t = 0.0;
            for (int w = 0; w < SM_WARPS; ++w) t += wred[w];
            red_s[slot] = t;
        }
        cluster.sync();
        double tot = 0.0;
        for (int o = 0; o < G.CL; ++o) tot += *cluster.map_shared_rank(red_s + slot, o);
        return tot;
    };

    // z = K_0^-1 r on interior points (lanes over modes), boundary rows of z stay zero
    auto precondition = [&]() {
        // x-transform of my interior lines: T[y][kx] = sum_x S[kx][x] r[y][x]
        for (int it = warp; it < (l1 - l0) * G.N; it += SM_WARPS) {
            const int ly = it / G.N, kx = it - ly * G.N;
            const int y = l0 + ly;
            float acc = 0.f;
            if (y >= 1 && y <= G.N) {
                const float* rr = r_s + (ly * G.NP + 1) * 32 + lane;
                const float* sr = S_s + kx * G.NS;
                for (int x = 0; x < G.N; ++x) acc = fmaf(sr[x], rr[x * 32], acc);
            }
            T_s[(ly * G.N + kx) * 32 + lane] = acc;
        }
        cluster.sync();
        // my columns kx in [k0, k1) from the owners of every interior line
        for (int it = warp; it < G.N * nk; it += SM_WARPS) {
            const int y1 = it / nk, kk = it - y1 * nk;  // interior line y1 + 1
            const int y = y1 + 1, o = owner_s[y];
            const float* src = cluster.map_shared_rank(T_s, o);
            Tl_s[(y1 * G.MAXK + kk) * 32 + lane] = src[((y - line_lo(o, G)) * G.N + k0 + kk) * 32 + lane];
        }
        __syncthreads();
        // U[ky][kx] = scale * sum_y S[ky][y] Tl[y][kx] ; V[y][kx] = sum_ky S[y][ky] U[ky][kx]
        for (int it = warp; it < G.N * nk; it += SM_WARPS) {
            const int ky = it / nk, kk = it - ky * nk;
            const float* sr = S_s + ky * G.NS;
            float acc = 0.f;
            for (int y1 = 0; y1 < G.N; ++y1) acc = fmaf(sr[y1], Tl_s[(y1 * G.MAXK + kk) * 32 + lane], acc);
            V_s[(ky * G.MAXK + kk) * 32 + lane] = acc * tb.scale[ky * G.N + k0 + kk];
        }
        __syncthreads();
        for (int it = warp; it < G.N * nk; it += SM_WARPS) {  // back along y, into Tl
            const int y1 = it / nk, kk = it - y1 * nk;
            const float* sr = S_s + y1 * G.NS;
            float acc = 0.f;
            for (int ky = 0; ky < G.N; ++ky) acc = fmaf(sr[ky], V_s[(ky * G.MAXK + kk) * 32 + lane], acc);
            Tl_s[(y1 * G.MAXK + kk) * 32 + lane] = acc;
        }
        cluster.sync();
        // all columns of my interior lines from their owners, then back along x
        for (int it = warp; it < (l1 - l0) * G.N; it += SM_WARPS) {
            const int ly = it / G.N, kx = it - ly * G.N;
            const int y = l0 + ly;
            float v = 0.f;
            if (y >= 1 && y <= G.N) {
                int o = 0;
                while (o + 1 < G.CL && col_lo(o + 1, G) <= kx) ++o;
                const float* src = cluster.map_shared_rank(Tl_s, o);
                v = src[((y - 1) * G.MAXK + (kx - col_lo(o, G))) * 32 + lane];
            }
            Vl_s[(ly * G.N + kx) * 32 + lane] = v;
        }
        __syncthreads();
        for (int it = warp; it < (l1 - l0) * G.N; it += SM_WARPS) {
            const int ly = it / G.N, x1 = it - ly * G.N;
            const int y = l0 + ly;
            if (y < 1 || y > G.N) continue;
            const float* sr = S_s + x1 * G.NS;
            const float* vr = Vl_s + ly * G.N * 32 + lane;
            float acc = 0.f;
            for (int kx = 0; kx < G.N; ++kx) acc = fmaf(sr[kx], vr[kx * 32], acc);
            z_s[(ly * G.NP + x1 + 1) * 32 + lane] = lv ? acc : 0.f;
        }
        __syncthreads();
    };

    // q = A p on my rows
    auto apply = [&]() -> double {
        double part = 0.0;
        for (int li = warp; li < nrow; li += SM_WARPS) {
            const int gi = row0 + li;
            float qv = 0.f;
            if (!bmask[gi]) {
                const float pi_ = p_s[li * 32 + lane];
                float w[SM_MAXM1];
#pragma unroll
                for (int m = 0; m < SM_MAXM1; ++m) w[m] = 0.f;
                for (int k = rowptr[gi]; k < rowptr[gi + 1]; ++k) {
                    const int j = col[k];
                    const int jy = j / G.NP, o = owner_s[jy];
                    const int lj = j - line_lo(o, G) * G.NP;
                    const float* pp = (o == me) ? p_s : cluster.map_shared_rank(p_s, o);
                    const float pj = pp[lj * 32 + lane];
                    const float u = G.diff ? pj - pi_ : pj;
                    const float* kv = vals + (size_t)k * G.M1P;
#pragma unroll
                    for (int m = 0; m < SM_MAXM1; ++m)
                        if (m < G.M1) w[m] = fmaf(__ldg(kv + m), u, w[m]);
                }
                qv = w[0];
#pragma unroll
                for (int m = 1; m < SM_MAXM1; ++m) {
                    if (m >= G.M1) break;
                    for (int sl = 0; sl < nslot_s[m]; ++sl) {  // warp-uniform count
                        const int at = (m * SM_MAXSLOT + sl) * 32 + lane;
                        const float v = __shfl_sync(0xffffffffu, w[m], src_s[at]);
                        qv = fmaf(g_s[at], v, qv);
                    }
                }
                if (!lv) qv = 0.f;
            }
            q_s[li * 32 + lane] = qv;
            part += (double)(p_s[li * 32 + lane] * qv);
        }
        return part;
    };

    // z = M^-1 r, rho = r'z, p = z
    precondition();
    double rz_loc = 0.0;
    for (int i = threadIdx.x; i < nrow * 32; i += SM_THREADS) {
        rz_loc += (double)(r_s[i] * z_s[i]);
        p_s[i] = z_s[i];
    }
    double rho = csum(rz_loc, 2);
    int iters = 0, status = SGFEM_OK;
    double rr = 0.0;
    {
        double rl = 0.0;
        for (int i = threadIdx.x; i < nrow * 32; i += SM_THREADS) rl += (double)(r_s[i] * r_s[i]);
        rr = csum(rl, 1);
    }
    if (!isfinite(rho)) status = SGFEM_ERR_NONFINITE;
    else if (!(rho > 0.0) && rr > tol2) status = SGFEM_ERR_BREAKDOWN;
    while (status == SGFEM_OK && rr > tol2) {
        if (iters >= maxit) {
            status = SGFEM_ERR_MAXIT;
            break;
        }
        cluster.sync();  // p complete in every CTA before the halo reads
        const double pq = csum(apply(), 0);
        if (!isfinite(pq)) { status = SGFEM_ERR_NONFINITE; break; }
        if (!(pq > 0.0)) { status = SGFEM_ERR_BREAKDOWN; break; }
        const double alpha = rho / pq;
        const float af = (float)alpha;
        double rl = 0.0;
        for (int i = threadIdx.x; i < nrow * 32; i += SM_THREADS) {
            const int li = i >> 5, c = i & 31;
            if (c < G.ld) x64[(size_t)(row0 + li) * G.ld + c] += alpha * (double)p_s[i];
            const float rv = fmaf(-af, q_s[i], r_s[i]);
            r_s[i] = rv;
            rl += (double)(rv * rv);
        }
        rr = csum(rl, 1);
        ++iters;
        if (!isfinite(rr)) { status = SGFEM_ERR_NONFINITE; break; }
        if (rr <= tol2) break;
        precondition();
        double zl = 0.0;
        for (int i = threadIdx.x; i < nrow * 32; i += SM_THREADS) zl += (double)(r_s[i] * z_s[i]);
        const double rho_new = csum(zl, 2);
        if (!isfinite(rho_new)) { status = SGFEM_ERR_NONFINITE; break; }
        if (!(rho_new > 0.0)) { status = SGFEM_ERR_BREAKDOWN; break; }
        const float bf = (float)(rho_new / rho);
        rho = rho_new;
        for (int i = threadIdx.x; i < nrow * 32; i += SM_THREADS) p_s[i] = fmaf(bf, p_s[i], z_s[i]);
    }
    cluster.sync();  // no CTA leaves while another may still read its shared memory
    if (me == 0 && threadIdx.x == 0) {
        scal->iters = iters;
        scal->status = status;
        scal->rr = rr;
        scal->done = 1;
    }
}

}  // namespace

struct SmallPCG {
    bool ok = false;
    std::string why = "not prepared";
    double a0 = 0.0;
    SmallGeom geom{};
    float* d_S = nullptr;
    float* d_scale = nullptr;
    int* d_nslot = nullptr;
    int* d_src = nullptr;
    float* d_g = nullptr;
    bool tables = false;  // coupling tables for the current G
    size_t smem = 0;
};

static void small_free_tables(SmallPCG* s) {
    if (s->d_nslot) cudaFree(s->d_nslot);
    if (s->d_src) cudaFree(s->d_src);
    if (s->d_g) cudaFree(s->d_g);
    s->d_nslot = nullptr;
    s->d_src = nullptr;
    s->d_g = nullptr;
    s->tables = false;
}

void sg_small_release(sgfem_context* ctx) {
    SmallPCG* s = ctx->small;
    if (!s) return;
    small_free_tables(s);
    if (s->d_S) cudaFree(s->d_S);
    if (s->d_scale) cudaFree(s->d_scale);
    delete s;
    ctx->small = nullptr;
}

void sg_small_invalidate(sgfem_context* ctx) {
    if (ctx->small) small_free_tables(ctx->small);
}

const char* sg_small_log(const sgfem_context* ctx) { return ctx->small ? ctx->small->why.c_str() : "not prepared"; }

static size_t small_smem(const SmallGeom& G) {
    const size_t RMAX = (size_t)G.MAXL * G.NP;
    size_t f = 4 * RMAX * 32 + (size_t)G.MAXL * G.N * 32 + 2 * (size_t)G.N * G.MAXK * 32 +
               (size_t)G.MAXL * G.N * 32 + (size_t)G.N * G.NS + ((G.NP + 3) & ~3) +
               (size_t)G.M1 * SM_MAXSLOT * 32 + (((size_t)G.M1 * SM_MAXSLOT * 32 + 1) & ~(size_t)1);
    return f * sizeof(float) + 4 * sizeof(double);
}

// at finalize (rowptr/col/val64 in device numbering): is K_0 on the interior rows a0 times
// the 5-point Laplacian of a power-of-two P1 lattice, with few enough modes and terms?
int sg_small_prepare(sgfem_context* ctx, const std::vector<int64_t>& rowptr, const std::vector<int32_t>& col,
                     const std::vector<double>& val64) {
    sg_small_release(ctx);
    SmallPCG* s = new SmallPCG();
    ctx->small = s;
    const char* env = getenv("SGFEM_SMALL");
    if (env && atoi(env) == 0) {
        s->why = "disabled (SGFEM_SMALL=0)";
        return SGFEM_OK;
    }
    const int NP = ctx->lat_np;
    if (!ctx->lattice || !ctx->lat_order || ctx->batched || (int64_t)NP * NP != ctx->n) {
        s->why = "needs a power-of-two P1 dof lattice";
        return SGFEM_OK;
    }
    if (ctx->ld > 32 || ctx->M1 > SM_MAXM1) {
        s->why = "more than 32 modes or 16 KLE terms";
        return SGFEM_OK;
    }
    const int M1 = ctx->M1;
    double a0 = -1.0;
    for (int64_t i = 0; i < ctx->n; ++i) {
        if (ctx->bmask_host[i]) continue;
        const int iy = (int)(i / NP), ix = (int)(i % NP);
        double d = 0.0;
        for (int64_t k = rowptr[i]; k < rowptr[i + 1]; ++k) {
            const int jy = col[k] / NP, jx = col[k] % NP;
            const double v = val64[(size_t)k * M1 + 0];
            const int dx = jx - ix, dy = jy - iy;
            if (dx == 0 && dy == 0) d = v;
        }
        if (a0 < 0.0) a0 = d / 4.0;
        if (!(a0 > 0.0) || std::fabs(d - 4.0 * a0) > 1e-12 * d) {
            s->why = "K_0 is not a0 times the 5-point Laplacian (diagonal)";
            return SGFEM_OK;
        }
        for (int64_t k = rowptr[i]; k < rowptr[i + 1]; ++k) {
            const int jy = col[k] / NP, jx = col[k] % NP;
            const double v = val64[(size_t)k * M1 + 0];
            const int dx = jx - ix, dy = jy - iy;
            const bool nb = std::abs(dx) + std::abs(dy) == 1;
            const double want = (dx == 0 && dy == 0) ? 4.0 * a0 : (nb ? -a0 : 0.0);
            // entries in boundary columns do not reach interior values (boundary rows of p are zero)
            if (ctx->bmask_host[col[k]]) continue;
            if (std::fabs(v - want) > 1e-12 * 4.0 * a0) {
                s->why = "K_0 is not a0 times the 5-point Laplacian";
                return SGFEM_OK;
            }
        }
        if (ctx->row_nnz_max > 64) break;
    }
    const int Nl = NP - 1, N = Nl - 1;
    SmallGeom G{};
    G.NP = NP;
    G.N = N;
    G.NS = (N + 3) & ~3;
    G.ld = (int)ctx->ld;
    G.M1 = M1;
    G.M1P = ctx->M1P;
    G.diff = ctx->rowsum_zero ? 1 : 0;
    // the largest cluster the device runs (16 non-portable, else 8) whose share fits
    size_t smem = 0;
    int CL = 0;
    const char* ecl = getenv("SGFEM_SMALL_CLUSTER");  // 8: the portable cluster size only
    const int clmax = ecl ? atoi(ecl) : 16;
    for (int c : {16, 8}) {
        if (c > clmax) continue;
        SmallGeom t = G;
        t.CL = c;
        t.MAXL = (NP + c - 1) / c;
        t.MAXK = (N + c - 1) / c;
        if (t.MAXL < 1 || t.MAXK < 1) continue;
        const size_t b = small_smem(t);
        if (b > 200 * 1024) continue;
        if (cudaFuncSetAttribute(k_small_pcg, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)b) != cudaSuccess ||
            (c > 8 && cudaFuncSetAttribute(k_small_pcg, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) !=
                          cudaSuccess)) {
            cudaGetLastError();
            continue;
        }
        cudaLaunchConfig_t cfg{};
        cudaLaunchAttribute at[1];
        at[0].id = cudaLaunchAttributeClusterDimension;
        at[0].val.clusterDim.x = c;
        at[0].val.clusterDim.y = 1;
        at[0].val.clusterDim.z = 1;
        cfg.gridDim = dim3(c);
        cfg.blockDim = dim3(SM_THREADS);
        cfg.dynamicSmemBytes = b;
        cfg.attrs = at;
        cfg.numAttrs = 1;
        int nclusters = 0;
        if (cudaOccupancyMaxActiveClusters(&nclusters, k_small_pcg, &cfg) != cudaSuccess || nclusters < 1) {
            cudaGetLastError();
            continue;
        }
        G = t;
        CL = c;
        smem = b;
        break;
    }
    if (!CL) {
        s->why = "no cluster shape fits";
        return SGFEM_OK;
    }
    std::vector<float> S((size_t)N * G.NS, 0.f), scale((size_t)N * N);
    const double pi = 3.14159265358979323846;
    for (int k = 1; k <= N; ++k)
        for (int x = 1; x <= N; ++x) S[(size_t)(k - 1) * G.NS + (x - 1)] = (float)(std::sqrt(2.0 / Nl) * std::sin(pi * k * x / Nl));
    auto lam = [&](int k) { const double sv = std::sin(pi * k / (2.0 * Nl)); return 4.0 * sv * sv; };
    for (int ky = 1; ky <= N; ++ky)
        for (int kx = 1; kx <= N; ++kx) scale[(size_t)(ky - 1) * N + (kx - 1)] = (float)(1.0 / (a0 * (lam(kx) + lam(ky))));
    if (cudaMalloc((void**)&s->d_S, S.size() * sizeof(float)) != cudaSuccess ||
        cudaMemcpy(s->d_S, S.data(), S.size() * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMalloc((void**)&s->d_scale, scale.size() * sizeof(float)) != cudaSuccess ||
        cudaMemcpy(s->d_scale, scale.data(), scale.size() * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess)
        return sg_fail(ctx, SGFEM_ERR_CUDA, "small PCG: table upload failed");
    s->a0 = a0;
    s->geom = G;
    s->smem = smem;
    s->ok = true;
    s->why = "one-cluster FP32 PCG: " + std::to_string(CL) + " CTAs, " + std::to_string(smem / 1024) +
             " KB shared memory each";
    return SGFEM_OK;
}

// coupling tables for the current G (built at the first use, again after a coupling update)
static int small_tables(sgfem_context* ctx, SmallPCG* s) {
    if (s->tables) return SGFEM_OK;
    const int P = (int)ctx->P, M1 = ctx->M1;
    std::vector<std::vector<std::vector<std::pair<int, float>>>> lst(M1, std::vector<std::vector<std::pair<int, float>>>(32));
    for (int mu = 0; mu < P; ++mu)
        for (int32_t e = ctx->h_combptr[mu]; e < ctx->h_combptr[mu + 1]; ++e) {
            const int32_t q = ctx->h_qtab[ctx->h_combq[e]];
            const int m = q >> 16, nu = q & 0xffff;
            lst[m][mu].push_back({nu, (float)ctx->h_combg[e]});
        }
    std::vector<int> nslot(M1, 0), src((size_t)M1 * SM_MAXSLOT * 32), gmax;
    std::vector<float> g((size_t)M1 * SM_MAXSLOT * 32, 0.f);
    for (int m = 0; m < M1; ++m)
        for (int L = 0; L < 32; ++L) {
            if ((int)lst[m][L].size() > SM_MAXSLOT) return SGFEM_ERR_UNSUPPORTED;
            nslot[m] = std::max(nslot[m], (int)lst[m][L].size());
            for (int t = 0; t < SM_MAXSLOT; ++t) {
                const size_t at = ((size_t)m * SM_MAXSLOT + t) * 32 + L;
                src[at] = t < (int)lst[m][L].size() ? lst[m][L][t].first : L;
                g[at] = t < (int)lst[m][L].size() ? lst[m][L][t].second : 0.f;
            }
        }
    if (cudaMalloc((void**)&s->d_nslot, nslot.size() * sizeof(int)) != cudaSuccess ||
        cudaMemcpy(s->d_nslot, nslot.data(), nslot.size() * sizeof(int), cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMalloc((void**)&s->d_src, src.size() * sizeof(int)) != cudaSuccess ||
        cudaMemcpy(s->d_src, src.data(), src.size() * sizeof(int), cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMalloc((void**)&s->d_g, g.size() * sizeof(float)) != cudaSuccess ||
        cudaMemcpy(s->d_g, g.data(), g.size() * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess)
        return SGFEM_ERR_CUDA;
    s->tables = true;
    return SGFEM_OK;
}

bool sg_small_usable(sgfem_context* ctx) {
    SmallPCG* s = ctx->small;
    if (!s || !s->ok || ctx->ld > 32 || ctx->M1 > SM_MAXM1) return false;
    if (small_tables(ctx, s) != SGFEM_OK) {
        s->ok = false;
        s->why = "couplings outside the one-cluster PCG's tables";
        return false;
    }
    return true;
}

// FP32 PCG on A d = r32 from d = 0 to ||r||^2 <= scal->tol2 (set before), d accumulated in
// FP64 into d64 (zero on entry); iterations and status come back in scal
int sg_small_pcg(sgfem_context* ctx, const float* r32, double* d64, int maxit, int* iters, int* status) {
    SmallPCG* s = ctx->small;
    SmallGeom G = s->geom;
    G.ld = (int)ctx->ld;
    SmallTabs tb{s->d_S, s->d_scale, s->d_nslot, s->d_src, s->d_g};
    // the function attributes are per process: set this context's shared-memory size
    SG_CUDA(ctx, cudaFuncSetAttribute(k_small_pcg, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)s->smem));
    if (G.CL > 8) SG_CUDA(ctx, cudaFuncSetAttribute(k_small_pcg, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
    cudaLaunchConfig_t cfg{};
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = G.CL;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.gridDim = dim3(G.CL);
    cfg.blockDim = dim3(SM_THREADS);
    cfg.dynamicSmemBytes = s->smem;
    cfg.stream = ctx->stream;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    SG_CUDA(ctx, cudaLaunchKernelEx(&cfg, k_small_pcg, (const int*)ctx->d_rowptr, (const int*)ctx->d_col,
                                    (const float*)ctx->d_val32p, (const unsigned char*)ctx->d_bmask, r32, d64,
                                    ctx->d_scal, tb, G, maxit));
    ctx->launches++;
    KrylovScalars* h = ctx->h_scal;
    SG_CUDA(ctx, cudaMemcpyAsync(h, ctx->d_scal, sizeof(KrylovScalars), cudaMemcpyDeviceToHost, ctx->stream));
    SG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    *iters = h->iters;
    *status = h->status;
    return SGFEM_OK;
}

extern "C" const char* sgfem_small_solve_log(const sgfem_context* ctx) {
    if (!ctx) return "null context";
    return sg_small_log(ctx);
}
