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
// memory, p with one halo line on each side.  Apply: a warp per row, all
// operands in shared memory; per row w_m = sum_j K_m[i,j] (p_j - p_i)
// (difference form, the diagonal left out) for every KLE term, then
// q_mu = w_0[mu] + sum g w_m[nu] with nu fetched by warp shuffles from the lane
// that owns it.  Preconditioner: x-transform of the CTA's lines, then CTA b
// transforms the columns kx of its share along y (scale, back along y), then the
// x-transform back of its lines; the two changes of ownership read the other
// CTAs' shared memory.  Dot products: per-warp partials, which every warp of
// every CTA sums in one fixed order (all CTAs take identical decisions).  The
// halo lines of p = z + beta p are formed by each CTA from the owners' z, so an
// iteration has four cluster barriers: the p'q sum, the two transposes of the
// preconditioner and the joint r'r, r'z sum.  The FP64 solution correction
// accumulates in shared memory (x += alpha p in FP64, as in the multi-launch
// solve) and is written out at the end.
#include <cooperative_groups.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "sgfem_internal.h"

namespace cg = cooperative_groups;

namespace {

constexpr int SM_THREADS = 512;
constexpr int SM_WARPS = SM_THREADS / 32;
constexpr int SM_MAXM1 = 16;   // KLE terms (M + 1) the kernel holds per row
constexpr int SM_MAXSLOT = 4;  // couplings per (term, output mode)
constexpr int SM_R = 4;        // transform outputs per warp item (they share the lane-strided loads)

struct SmallGeom {
    int NP;      // lattice points per line (Nl + 1)
    int N;       // interior points per line (Nl - 1)
    int NS;      // row stride of the sine matrix (N rounded up to 4)
    int ld, M1, M1P;
    int KS;      // stride of a staged nonzero's KLE values (M1 rounded up to 2)
    int CL;      // CTAs in the cluster
    int MAXL;    // lines per CTA (most)
    int MAXK;    // transform columns per CTA (most)
    int TMAX;    // staged nonzeros per row (most; the diagonal is left out in difference form)
    int diff;
};

struct SmallTabs {
    const float* S;       // N x NS, S[k][x] (symmetric)
    const float* scale;   // N x N, 1 / (a0 (lam_ky + lam_kx)), [ky][kx]
    const int* nslot;     // [1]: couplings per (term, output mode), most over all terms and modes
    const int2* cg;       // [SM_MAXSLOT][M1][32]: {source lane, bits of g} (g = 0 for padding)
};

// float offsets of the shared-memory arrays, each start 16-byte aligned
struct SmallLayout {
    int xh, xl, pe, r, q, z, T, Tl, V, sc, S, kv, own, cown, cj, cg, red, total;
};

__host__ __device__ inline int small_take(int& o, int nfloats) {
    const int at = o;
    o += (nfloats + 3) & ~3;
    return at;
}

__host__ __device__ inline SmallLayout small_layout(const SmallGeom& G) {
    SmallLayout L{};
    int o = 0;
    const int RMAX = G.MAXL * G.NP;
    L.xh = small_take(o, RMAX * G.ld);               // [RMAX][ld]: the correction of my rows, high part
    L.xl = small_take(o, RMAX * G.ld);               // and low part (x = xh + xl)
    L.pe = small_take(o, (RMAX + 2 * G.NP) * 32);     // p, lines l0 - 1 .. l0 + MAXL
    L.r = small_take(o, RMAX * 32);
    L.q = small_take(o, RMAX * 32);
    L.z = small_take(o, RMAX * 32);
    L.T = small_take(o, G.MAXL * G.N * 32);           // [MAXL][N][32]: x-transform of my lines
    L.Tl = small_take(o, G.N * G.MAXK * 32);          // [N][MAXK][32]: my columns, all lines
    L.V = small_take(o, G.N * G.MAXK * 32);           // [N][MAXK][32]: my columns after y and scale
    L.sc = small_take(o, G.N * G.MAXK);               // [N][MAXK]: preconditioner scale of my columns
    L.S = small_take(o, G.N * G.NS);                  // [N][NS]
    L.kv = small_take(o, RMAX * G.TMAX * G.KS);       // [RMAX][TMAX][KS]: my rows' KLE values
    L.own = small_take(o, G.NP);                      // [NP]: owner CTA << 16 | line index in the owner
    L.cown = small_take(o, G.N);                      // [N]: the same for transform columns
    L.cj = small_take(o, RMAX * G.TMAX);              // [RMAX][TMAX]: row of pe of each nonzero (-1: boundary row)
    L.cg = small_take(o, SM_MAXSLOT * G.M1 * 32 * 2); // int2 [SM_MAXSLOT][M1][32]
    L.red = small_take(o, 3 * SM_WARPS);              // [3][SM_WARPS]: p'q, r'r, r'z partials
    L.total = o;
    return L;
}

// out[r] = sum_k S[kr + r][k] * b[k * bs] for r < SM_R (rows clamped to N - 1: their outputs are
// not stored), S rows 16-byte aligned and broadcast, b lane-strided and shared by the SM_R sums
__device__ __forceinline__ void dotR(const float* __restrict__ S_s, int NS, int kr, int N,
                                     const float* __restrict__ b, int bs, float out[SM_R]) {
    const float* a[SM_R];
#pragma unroll
    for (int r = 0; r < SM_R; ++r) {
        a[r] = S_s + min(kr + r, N - 1) * NS;
        out[r] = 0.f;
    }
    int k = 0;
    for (; k + 4 <= N; k += 4) {
        const float b0 = b[k * bs], b1 = b[(k + 1) * bs], b2 = b[(k + 2) * bs], b3 = b[(k + 3) * bs];
#pragma unroll
        for (int r = 0; r < SM_R; ++r) {
            const float4 av = *reinterpret_cast<const float4*>(a[r] + k);
            out[r] = fmaf(av.x, b0, out[r]);
            out[r] = fmaf(av.y, b1, out[r]);
            out[r] = fmaf(av.z, b2, out[r]);
            out[r] = fmaf(av.w, b3, out[r]);
        }
    }
    for (; k < N; ++k) {
        const float bk = b[k * bs];
#pragma unroll
        for (int r = 0; r < SM_R; ++r) out[r] = fmaf(a[r][k], bk, out[r]);
    }
}

// (xh, xl) += (ph, pl) in double-FP32 arithmetic (Knuth's TwoSum of the high parts, then
// the low parts, renormalised)
__device__ __forceinline__ void df_add(float& xh, float& xl, float ph, float pl) {
    const float s = xh + ph;
    const float bv = s - xh;
    const float e = (xh - (s - bv)) + (ph - bv);
    const float t = e + (xl + pl);
    xh = s + t;
    xl = t - (xh - s);
}

// first line / transform column of CTA b (b <= CL; the products stay far below 2^31)
__device__ __forceinline__ int line_lo(int b, const SmallGeom& G) { return b * G.NP / G.CL; }
__device__ __forceinline__ int col_lo(int b, const SmallGeom& G) { return b * G.N / G.CL; }

// q = A p on my rows for M1 KLE terms (w_m in registers); returns this thread's p'q partial.
// Rows are padded to TMAX nonzeros with zero values (no data-dependent exit), couplings to
// nsl slots per term with g = 0.
template <int M1>
__device__ __forceinline__ float apply_rows(const int* __restrict__ cj_s, const float* __restrict__ kv_s,
                                            const float* __restrict__ pe_s, const float* __restrict__ p_s,
                                            float* __restrict__ q_s, const int2* __restrict__ cg_s, int nsl,
                                            int nrow, int warp, int lane, const SmallGeom& G) {
    constexpr int KS = (M1 + 1) & ~1;
    const bool lv = lane < G.ld;
    float part = 0.f;
    for (int li = warp; li < nrow; li += SM_WARPS) {
        float qv = 0.f;
        const int* cr = cj_s + li * G.TMAX;
        const float pi_ = p_s[li * 32 + lane];
        if (cr[0] >= 0) {  // warp-uniform: not a boundary row
            float w[M1];
#pragma unroll
            for (int m = 0; m < M1; ++m) w[m] = 0.f;
            const float* kv = kv_s + (size_t)li * G.TMAX * KS;
#pragma unroll 2
            for (int t = 0; t < G.TMAX; ++t) {
                const float pj = pe_s[cr[t] * 32 + lane];
                const float u = G.diff ? pj - pi_ : pj;
#pragma unroll
                for (int m = 0; m + 1 < M1; m += 2) {
                    const float2 v = *reinterpret_cast<const float2*>(kv + t * KS + m);
                    w[m] = fmaf(v.x, u, w[m]);
                    w[m + 1] = fmaf(v.y, u, w[m + 1]);
                }
                if (M1 & 1) w[M1 - 1] = fmaf(kv[t * KS + M1 - 1], u, w[M1 - 1]);
            }
            qv = w[0];
            for (int sl = 0; sl < nsl; ++sl) {  // warp-uniform count; the terms of a slot are independent
#pragma unroll
                for (int m = 1; m < M1; ++m) {
                    const int2 e = cg_s[(sl * M1 + m) * 32 + lane];
                    const float v = __shfl_sync(0xffffffffu, w[m], e.x);
                    qv = fmaf(__int_as_float(e.y), v, qv);
                }
            }
            if (!lv) qv = 0.f;
        }
        q_s[li * 32 + lane] = qv;
        part = fmaf(pi_, qv, part);
    }
    return part;
}

// the same for any M1 <= SM_MAXM1 at run time (the term loops run to SM_MAXM1 behind a
// warp-uniform guard): one code body for the counts above those specialised
__device__ __forceinline__ float apply_rows_any(const int* __restrict__ cj_s, const float* __restrict__ kv_s,
                                                const float* __restrict__ pe_s, const float* __restrict__ p_s,
                                                float* __restrict__ q_s, const int2* __restrict__ cg_s, int nsl,
                                                int nrow, int warp, int lane, const SmallGeom& G) {
    const int M1 = G.M1, KS = G.KS;
    const bool lv = lane < G.ld;
    float part = 0.f;
    for (int li = warp; li < nrow; li += SM_WARPS) {
        float qv = 0.f;
        const int* cr = cj_s + li * G.TMAX;
        const float pi_ = p_s[li * 32 + lane];
        if (cr[0] >= 0) {  // warp-uniform: not a boundary row
            float w[SM_MAXM1];
#pragma unroll
            for (int m = 0; m < SM_MAXM1; ++m) w[m] = 0.f;
            const float* kv = kv_s + (size_t)li * G.TMAX * KS;
            for (int t = 0; t < G.TMAX; ++t) {
                const float pj = pe_s[cr[t] * 32 + lane];
                const float u = G.diff ? pj - pi_ : pj;
#pragma unroll
                for (int m = 0; m < SM_MAXM1; m += 2) {
                    if (m < M1) {  // KS is even and the staged values are zero beyond M1
                        const float2 v = *reinterpret_cast<const float2*>(kv + t * KS + m);
                        w[m] = fmaf(v.x, u, w[m]);
                        w[m + 1] = fmaf(v.y, u, w[m + 1]);
                    }
                }
            }
            qv = w[0];
            for (int sl = 0; sl < nsl; ++sl) {
#pragma unroll
                for (int m = 1; m < SM_MAXM1; ++m) {
                    if (m < M1) {
                        const int2 e = cg_s[(sl * M1 + m) * 32 + lane];
                        const float v = __shfl_sync(0xffffffffu, w[m], e.x);
                        qv = fmaf(__int_as_float(e.y), v, qv);
                    }
                }
            }
            if (!lv) qv = 0.f;
        }
        q_s[li * 32 + lane] = qv;
        part = fmaf(pi_, qv, part);
    }
    return part;
}

__global__ void __launch_bounds__(SM_THREADS, 1)
k_small_pcg(const int* __restrict__ rowptr, const int* __restrict__ col, const float* __restrict__ vals,
            const unsigned char* __restrict__ bmask, const float* __restrict__ rin, double* __restrict__ x64,
            KrylovScalars* __restrict__ scal, SmallTabs tb, SmallGeom G, int maxit) {
    cg::cluster_group cluster = cg::this_cluster();
    const int me = (int)cluster.block_rank();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    extern __shared__ __align__(16) float sm[];
    const SmallLayout L = small_layout(G);
    const int RMAX = G.MAXL * G.NP;
    float* xh_s = sm + L.xh;
    float* xl_s = sm + L.xl;
    float* pe_s = sm + L.pe;
    float* p_s = pe_s + G.NP * 32;  // my rows; halo line l0 - 1 before, l1 after
    float* r_s = sm + L.r;
    float* q_s = sm + L.q;
    float* z_s = sm + L.z;
    float* T_s = sm + L.T;
    float* Tl_s = sm + L.Tl;
    float* V_s = sm + L.V;
    // all columns of my lines; shares T_s's storage (T_s is read by the other CTAs only
    // before the second barrier of an application, Vl_s written after it)
    float* Vl_s = T_s;
    float* sc_s = sm + L.sc;
    float* S_s = sm + L.S;
    float* kv_s = sm + L.kv;
    int* owner_s = reinterpret_cast<int*>(sm + L.own);
    int* cown_s = reinterpret_cast<int*>(sm + L.cown);
    int* cj_s = reinterpret_cast<int*>(sm + L.cj);
    int2* cg_s = reinterpret_cast<int2*>(sm + L.cg);
    float* red_s = sm + L.red;

    const int l0 = line_lo(me, G), l1 = line_lo(me + 1, G);
    const int nl = l1 - l0;
    const int nrow = nl * G.NP;
    const int row0 = l0 * G.NP;
    const int k0 = col_lo(me, G), k1 = col_lo(me + 1, G);
    const int nk = k1 - k0;
    const int ng = (G.N + SM_R - 1) / SM_R;  // groups of SM_R transform outputs along a line
    const bool lv = lane < G.ld;
    const int nsl = tb.nslot[0];
    for (int i = threadIdx.x; i < G.N * G.NS; i += SM_THREADS) S_s[i] = tb.S[i];
    for (int i = threadIdx.x; i < G.N * nk; i += SM_THREADS) {
        const int ky = i / nk, kk = i - ky * nk;
        sc_s[ky * G.MAXK + kk] = tb.scale[ky * G.N + k0 + kk];
    }
    for (int i = threadIdx.x; i < RMAX * G.ld; i += SM_THREADS) {
        xh_s[i] = 0.f;
        xl_s[i] = 0.f;
    }
    for (int y = threadIdx.x; y < G.NP; y += SM_THREADS) {
        int o = 0;
        while (o + 1 < G.CL && line_lo(o + 1, G) <= y) ++o;
        owner_s[y] = o << 16 | (y - line_lo(o, G));
    }
    for (int kx = threadIdx.x; kx < G.N; kx += SM_THREADS) {
        int o = 0;
        while (o + 1 < G.CL && col_lo(o + 1, G) <= kx) ++o;
        cown_s[kx] = o << 16 | (kx - col_lo(o, G));
    }
    for (int i = threadIdx.x; i < (RMAX + 2 * G.NP) * 32; i += SM_THREADS) pe_s[i] = 0.f;
    for (int i = threadIdx.x; i < RMAX * 32; i += SM_THREADS) {
        const int li = i >> 5, c = i & 31;
        r_s[i] = (li < nrow && c < G.ld) ? rin[(size_t)(row0 + li) * G.ld + c] : 0.f;
        q_s[i] = 0.f;
        z_s[i] = 0.f;
    }
    // my rows' nonzeros, one thread per row: their row in the halo-extended p (lines
    // l0 - 1 .. l1) and KLE values, in difference form without the diagonal; padded to
    // TMAX with zero values (at row 0 of p); a boundary row is marked by -1
    for (int li = threadIdx.x; li < RMAX; li += SM_THREADS) {
        int cnt = 0;
        const bool interior = li < nrow && !bmask[row0 + li];
        if (interior) {
            const int gi = row0 + li;
            for (int k = rowptr[gi]; k < rowptr[gi + 1] && cnt < G.TMAX; ++k) {
                const int j = col[k];
                if (G.diff && j == gi) continue;
                const int at = li * G.TMAX + cnt;
                cj_s[at] = (j / G.NP - (l0 - 1)) * G.NP + j % G.NP;
                for (int m = 0; m < G.KS; ++m) kv_s[(size_t)at * G.KS + m] = m < G.M1 ? vals[(size_t)k * G.M1P + m] : 0.f;
                ++cnt;
            }
        }
        for (; cnt < G.TMAX; ++cnt) {
            const int at = li * G.TMAX + cnt;
            cj_s[at] = (interior || cnt > 0) ? 0 : -1;
            for (int m = 0; m < G.KS; ++m) kv_s[(size_t)at * G.KS + m] = 0.f;
        }
    }
    for (int i = threadIdx.x; i < SM_MAXSLOT * G.M1 * 32; i += SM_THREADS) cg_s[i] = tb.cg[i];
    __syncthreads();
    const float tol2 = (float)scal->tol2;
    const int nred = G.CL * SM_WARPS;

    // cluster-wide FP32 sums of per-thread values: warp sums into red_s, one cluster barrier,
    // then every warp adds the CL x SM_WARPS partials in one fixed order (lane e sums
    // entries e, e + 32, ...; then a butterfly), so every thread of every CTA holds the
    // same totals.  A slot is written again only after a later cluster barrier.
    auto wsum = [&](float v) {
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        return v;
    };
    auto gather = [&](int slot) {
        float t = 0.f;
        for (int e = lane; e < nred; e += 32)
            t += *cluster.map_shared_rank(red_s + slot * SM_WARPS + (e & (SM_WARPS - 1)), e / SM_WARPS);
        for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
        return t;
    };
    auto csum1 = [&](float v, int slot) -> float {
        v = wsum(v);
        if (lane == 0) red_s[slot * SM_WARPS + warp] = v;
        cluster.sync();
        return gather(slot);
    };
    auto csum2 = [&](float a, float b, float& ta, float& tb2) {
        a = wsum(a);
        b = wsum(b);
        if (lane == 0) {
            red_s[1 * SM_WARPS + warp] = a;
            red_s[2 * SM_WARPS + warp] = b;
        }
        cluster.sync();
        ta = gather(1);
        tb2 = gather(2);
    };

    // z = K_0^-1 r on interior points (lanes over modes), boundary rows of z stay zero
    auto precondition = [&]() {
        float o4[SM_R];
        // x-transform of my interior lines: T[y][kx] = sum_x S[kx][x] r[y][x]
        for (int it = warp; it < nl * ng; it += SM_WARPS) {
            const int ly = it / ng, kx = (it - ly * ng) * SM_R;
            const int y = l0 + ly;
            if (y >= 1 && y <= G.N) dotR(S_s, G.NS, kx, G.N, r_s + (ly * G.NP + 1) * 32 + lane, 32, o4);
            else for (int r = 0; r < SM_R; ++r) o4[r] = 0.f;
#pragma unroll
            for (int r = 0; r < SM_R; ++r)
                if (kx + r < G.N) T_s[(ly * G.N + kx + r) * 32 + lane] = o4[r];
        }
        cluster.sync();
        // my columns kx in [k0, k1) from the owners of every interior line
        for (int it = warp; it < G.N * nk; it += SM_WARPS) {
            const int y1 = it / nk, kk = it - y1 * nk;  // interior line y1 + 1
            const int ow = owner_s[y1 + 1];
            const float* src = cluster.map_shared_rank(T_s, ow >> 16);
            Tl_s[(y1 * G.MAXK + kk) * 32 + lane] = src[((ow & 0xffff) * G.N + k0 + kk) * 32 + lane];
        }
        __syncthreads();
        // U[ky][kx] = scale * sum_y S[ky][y] Tl[y][kx] ; V[y][kx] = sum_ky S[y][ky] U[ky][kx]
        for (int it = warp; it < ng * nk; it += SM_WARPS) {
            const int kg = it / nk, kk = it - kg * nk, ky = kg * SM_R;
            dotR(S_s, G.NS, ky, G.N, Tl_s + kk * 32 + lane, G.MAXK * 32, o4);
#pragma unroll
            for (int r = 0; r < SM_R; ++r)
                if (ky + r < G.N) V_s[((ky + r) * G.MAXK + kk) * 32 + lane] = o4[r] * sc_s[(ky + r) * G.MAXK + kk];
        }
        __syncthreads();
        for (int it = warp; it < ng * nk; it += SM_WARPS) {  // back along y, into Tl
            const int yg = it / nk, kk = it - yg * nk, y1 = yg * SM_R;
            dotR(S_s, G.NS, y1, G.N, V_s + kk * 32 + lane, G.MAXK * 32, o4);
#pragma unroll
            for (int r = 0; r < SM_R; ++r)
                if (y1 + r < G.N) Tl_s[((y1 + r) * G.MAXK + kk) * 32 + lane] = o4[r];
        }
        cluster.sync();
        // all columns of my interior lines from their owners, then back along x
        for (int it = warp; it < nl * G.N; it += SM_WARPS) {
            const int ly = it / G.N, kx = it - ly * G.N;
            const int y = l0 + ly;
            float v = 0.f;
            if (y >= 1 && y <= G.N) {
                const int ow = cown_s[kx];
                const float* src = cluster.map_shared_rank(Tl_s, ow >> 16);
                v = src[((y - 1) * G.MAXK + (ow & 0xffff)) * 32 + lane];
            }
            Vl_s[(ly * G.N + kx) * 32 + lane] = v;
        }
        __syncthreads();
        for (int it = warp; it < nl * ng; it += SM_WARPS) {
            const int ly = it / ng, x1 = (it - ly * ng) * SM_R;
            const int y = l0 + ly;
            if (y < 1 || y > G.N) continue;
            dotR(S_s, G.NS, x1, G.N, Vl_s + ly * G.N * 32 + lane, 32, o4);
#pragma unroll
            for (int r = 0; r < SM_R; ++r)
                if (x1 + r < G.N) z_s[(ly * G.NP + x1 + r + 1) * 32 + lane] = lv ? o4[r] : 0.f;
        }
        __syncthreads();
    };

    // p = z + bf p on my rows and on the halo lines l0 - 1 and l1, whose z comes from the
    // owners: complete since the last cluster barrier, and not rewritten before the owner's
    // next preconditioner, which starts after the next cluster barrier
    const int hy0 = l0 - 1, hy1 = l1;
    const bool h0 = nrow > 0 && hy0 >= 0, h1 = nrow > 0 && hy1 < G.NP;
    const float* hz0 = h0 ? cluster.map_shared_rank(z_s, owner_s[hy0] >> 16) + (size_t)(owner_s[hy0] & 0xffff) * G.NP * 32 : nullptr;
    const float* hz1 = h1 ? cluster.map_shared_rank(z_s, owner_s[hy1] >> 16) + (size_t)(owner_s[hy1] & 0xffff) * G.NP * 32 : nullptr;
    float* hp1 = pe_s + (size_t)(hy1 - hy0) * G.NP * 32;
    auto update_p = [&](float bf) {
        for (int i = threadIdx.x; i < nrow * 32; i += SM_THREADS) p_s[i] = fmaf(bf, p_s[i], z_s[i]);
#pragma unroll 4
        for (int i = threadIdx.x; i < G.NP * 32; i += SM_THREADS) {
            const float z0 = h0 ? hz0[i] : 0.f, z1 = h1 ? hz1[i] : 0.f;
            if (h0) pe_s[i] = fmaf(bf, pe_s[i], z0);
            if (h1) hp1[i] = fmaf(bf, hp1[i], z1);
        }
    };

    auto apply = [&]() -> float {
        switch (G.M1) {
#define SM_APPLY(k) \
    case k: return apply_rows<k>(cj_s, kv_s, pe_s, p_s, q_s, cg_s, nsl, nrow, warp, lane, G);
            SM_APPLY(1) SM_APPLY(2) SM_APPLY(3) SM_APPLY(4) SM_APPLY(5) SM_APPLY(6) SM_APPLY(7) SM_APPLY(8)
#undef SM_APPLY
            default: return apply_rows_any(cj_s, kv_s, pe_s, p_s, q_s, cg_s, nsl, nrow, warp, lane, G);
        }
    };

    // z = M^-1 r, rho = r'z, p = z
    precondition();
    float rr = 0.f, rho = 0.f;
    {
        float rl = 0.f, zl = 0.f;
        for (int i = threadIdx.x; i < nrow * 32; i += SM_THREADS) {
            rl = fmaf(r_s[i], r_s[i], rl);
            zl = fmaf(r_s[i], z_s[i], zl);
        }
        csum2(rl, zl, rr, rho);
    }
    int iters = 0, status = SGFEM_OK;
    float bf = 0.f;  // p = z + 0 p (p and its halo start at zero)
    if (!isfinite(rho) || !isfinite(rr)) status = SGFEM_ERR_NONFINITE;
    else if (!(rho > 0.f) && rr > tol2) status = SGFEM_ERR_BREAKDOWN;
    while (status == SGFEM_OK && rr > tol2) {
        if (iters >= maxit) {
            status = SGFEM_ERR_MAXIT;
            break;
        }
        update_p(bf);
        __syncthreads();
        const float pq = csum1(apply(), 0);
        if (!isfinite(pq)) { status = SGFEM_ERR_NONFINITE; break; }
        if (!(pq > 0.f)) { status = SGFEM_ERR_BREAKDOWN; break; }
        const float af = rho / pq;
        for (int i = threadIdx.x; i < nrow * 32; i += SM_THREADS) {
            const float pv = p_s[i];
            r_s[i] = fmaf(-af, q_s[i], r_s[i]);
            const int c = i & 31;
            if (c < G.ld) {  // x += af p with the product's rounding error kept (FMA), in double-FP32
                const int at = (i >> 5) * G.ld + c;
                const float ph = af * pv;
                df_add(xh_s[at], xl_s[at], ph, fmaf(af, pv, -ph));
            }
        }
        __syncthreads();
        // z for the next direction (wasted once, at convergence), then r'r and r'z in one sum
        precondition();
        float rl = 0.f, zl = 0.f;
        for (int i = threadIdx.x; i < nrow * 32; i += SM_THREADS) {
            rl = fmaf(r_s[i], r_s[i], rl);
            zl = fmaf(r_s[i], z_s[i], zl);
        }
        float rho_new;
        csum2(rl, zl, rr, rho_new);
        ++iters;
        if (!isfinite(rr)) { status = SGFEM_ERR_NONFINITE; break; }
        if (rr <= tol2) break;
        if (!isfinite(rho_new)) { status = SGFEM_ERR_NONFINITE; break; }
        if (!(rho_new > 0.f)) { status = SGFEM_ERR_BREAKDOWN; break; }
        bf = rho_new / rho;
        rho = rho_new;
    }
    // a failed solve (breakdown, non-finite values) returns a zero correction, so the
    // caller's iterate and residual stay those of the previous refinement step
    const bool keep = status == SGFEM_OK || status == SGFEM_ERR_MAXIT;
    for (int i = threadIdx.x; i < nrow * G.ld; i += SM_THREADS)
        x64[(size_t)row0 * G.ld + i] = keep ? (double)xh_s[i] + (double)xl_s[i] : 0.0;
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
    int* d_cg = nullptr;  // int2 {source lane, bits of g}
    bool tables = false;  // coupling tables for the current G
    size_t smem = 0;
    long long launches = 0;
    std::string log;
};

static void small_free_tables(SmallPCG* s) {
    if (s->d_nslot) cudaFree(s->d_nslot);
    if (s->d_cg) cudaFree(s->d_cg);
    s->d_nslot = nullptr;
    s->d_cg = nullptr;
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

const char* sg_small_log(const sgfem_context* ctx) {
    SmallPCG* s = ctx->small;
    if (!s) return "not prepared";
    s->log = s->why;
    if (s->ok) s->log += "; launches: " + std::to_string(s->launches);
    return s->log.c_str();
}

static size_t small_smem(const SmallGeom& G) { return (size_t)small_layout(G).total * sizeof(float); }

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
    if (ctx->win_hy > 1) {  // the apply reads one halo line on each side
        s->why = "couplings beyond the neighbouring lattice lines";
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
    G.KS = (M1 + 1) & ~1;
    G.diff = ctx->rowsum_zero ? 1 : 0;
    // staged nonzeros per interior row: in difference form the diagonal contributes nothing
    G.TMAX = 1;
    for (int64_t i = 0; i < ctx->n; ++i) {
        if (ctx->bmask_host[i]) continue;
        int c = 0;
        for (int64_t k = rowptr[i]; k < rowptr[i + 1]; ++k) c += !(G.diff && col[k] == i);
        G.TMAX = std::max(G.TMAX, c);
    }
    if (G.TMAX > 16) {
        s->why = "rows with more than 16 nonzeros";
        return SGFEM_OK;
    }
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
        if (b > 220 * 1024) continue;
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
    // slot-major [SM_MAXSLOT][M1][32]; the kernel runs the most slots any term m >= 1 needs.
    // The lists hold the terms m >= 1 only: K_0 acts on every mode alone (q = w_0 + ...)
    std::vector<int> nslot(1, 0), cgt((size_t)SM_MAXSLOT * M1 * 32 * 2);
    for (int m = 0; m < M1; ++m)
        for (int L = 0; L < 32; ++L) {
            if ((int)lst[m][L].size() > SM_MAXSLOT) return SGFEM_ERR_UNSUPPORTED;
            if (m > 0) nslot[0] = std::max(nslot[0], (int)lst[m][L].size());
            for (int t = 0; t < SM_MAXSLOT; ++t) {
                const size_t at = ((size_t)t * M1 + m) * 32 + L;
                const float g = t < (int)lst[m][L].size() ? lst[m][L][t].second : 0.f;
                cgt[2 * at] = t < (int)lst[m][L].size() ? lst[m][L][t].first : L;
                std::memcpy(&cgt[2 * at + 1], &g, sizeof(float));
            }
        }
    if (cudaMalloc((void**)&s->d_nslot, nslot.size() * sizeof(int)) != cudaSuccess ||
        cudaMemcpy(s->d_nslot, nslot.data(), nslot.size() * sizeof(int), cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMalloc((void**)&s->d_cg, cgt.size() * sizeof(int)) != cudaSuccess ||
        cudaMemcpy(s->d_cg, cgt.data(), cgt.size() * sizeof(int), cudaMemcpyHostToDevice) != cudaSuccess)
        return SGFEM_ERR_CUDA;
    s->tables = true;
    return SGFEM_OK;
}

// the shared memory of a launch for the context's current mode count (the x rows are ld wide)
static size_t small_launch_smem(const sgfem_context* ctx, const SmallPCG* s) {
    SmallGeom G = s->geom;
    G.ld = (int)ctx->ld;
    return small_smem(G);
}

bool sg_small_usable(sgfem_context* ctx) {
    SmallPCG* s = ctx->small;
    if (!s || !s->ok || ctx->ld > 32 || ctx->M1 > SM_MAXM1) return false;
    if (small_launch_smem(ctx, s) > 220 * 1024) {  // the mode count grew past the shared memory
        s->ok = false;
        s->why = "no cluster shape fits the grown mode count";
        return false;
    }
    if (small_tables(ctx, s) != SGFEM_OK) {
        s->ok = false;
        s->why = "couplings outside the one-cluster PCG's tables";
        return false;
    }
    return true;
}

// FP32 PCG on A d = r32 from d = 0 to ||r||^2 <= scal->tol2 (set before), d accumulated in
// FP64 into d64 (zero on entry; zero again if the solve fails).  The launch and the copy of
// the scalars to the host are queued on the context's stream without a wait: the caller
// reads iterations and status with sg_small_pcg_result after its next synchronisation.
int sg_small_pcg_launch(sgfem_context* ctx, const float* r32, double* d64, int maxit) {
    SmallPCG* s = ctx->small;
    SmallGeom G = s->geom;
    G.ld = (int)ctx->ld;
    SmallTabs tb{s->d_S, s->d_scale, s->d_nslot, reinterpret_cast<const int2*>(s->d_cg)};
    // sized for the geometry passed below (the layout the kernel computes from it)
    const size_t smem = small_smem(G);
    if (smem != small_launch_smem(ctx, s) || smem > 220 * 1024)
        return sg_fail(ctx, SGFEM_ERR_UNSUPPORTED, "small PCG: shared memory does not fit the mode count");
    // the function attributes are per process: set this context's shared-memory size
    SG_CUDA(ctx, cudaFuncSetAttribute(k_small_pcg, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    if (G.CL > 8) SG_CUDA(ctx, cudaFuncSetAttribute(k_small_pcg, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
    cudaLaunchConfig_t cfg{};
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = G.CL;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.gridDim = dim3(G.CL);
    cfg.blockDim = dim3(SM_THREADS);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = ctx->stream;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    SG_CUDA(ctx, cudaLaunchKernelEx(&cfg, k_small_pcg, (const int*)ctx->d_rowptr, (const int*)ctx->d_col,
                                    (const float*)ctx->d_val32p, (const unsigned char*)ctx->d_bmask, r32, d64,
                                    ctx->d_scal, tb, G, maxit));
    ctx->launches++;
    s->launches++;
    SG_CUDA(ctx, cudaMemcpyAsync(ctx->h_scal, ctx->d_scal, sizeof(KrylovScalars), cudaMemcpyDeviceToHost, ctx->stream));
    return SGFEM_OK;
}

void sg_small_pcg_result(const sgfem_context* ctx, int* iters, int* status) {
    *iters = ctx->h_scal->iters;
    *status = ctx->h_scal->status;
}

extern "C" const char* sgfem_small_solve_log(const sgfem_context* ctx) {
    if (!ctx) return "null context";
    return sg_small_log(ctx);
}
