// K8: many independent SG problems solved together on sm_103a.
//
// Each problem is the SG system of solve_primal! (src/modelproblems/
// solvers_poisson_primal.jl:130-169) on its own mesh, coefficient length M and
// multi-index set: Y_mu = K_0 X_mu + sum_{m,nu} G[(m-1)P+mu,nu] K_m X_nu with
// Dirichlet rows zeroed, b = e_1 (x) b0.  All problems advance through one
// Jacobi-preconditioned CG in lock step: every phase of an iteration (apply,
// alpha, update, preconditioner, beta, direction) is one launch covering all
// problems, and a batch of iterations is captured once in a CUDA graph and
// replayed; converged problems skip their blocks.
//
// Work split: problem p owns the contiguous block range [blk0, blk0 + nblk) of
// every batch kernel (block counts proportional to the problem's apply work),
// so each block's reduction partial belongs to one problem and the per-problem
// sums are fixed-order reductions over that range (bitwise reproducible).
// The apply is the pair-gather of the single-problem generic kernel with the
// problem's tables read from a descriptor; its launch shape (warps per block,
// pairs per lane, blocks) is chosen at finalize by timing the candidates
// (autotuner).  FP64 throughout.
#include <sys/stat.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>

#include "sgfem_internal.h"

struct BProb {
    int n, P, ld, M1, Qn;
    int blk0, nblk;
    long long voff;               // offset of the problem's vectors (n * ld values)
    const int* rowptr;
    const int* col;
    const double* vals;           // [nnz][M1]
    const unsigned char* bmask;
    const double* dinv;           // 0 on Dirichlet rows
    const int* qtab;              // m << 16 | nu
    const int* combptr;
    const int* combq;
    const double* combg;
    const float* vals32;          // FP32 copies for the inner PCG of the mixed solve
    const float* combg32;
    const float* dinv32;
    // column-slot form of the apply (k_bapply_cols): passes over virtual groups of 32
    // columns, each lane taking its column's KLE terms from the lanes that hold them
    int npass;                    // FP32 passes
    const int4* cpass;            // FP32 passes: (kind, first virtual group, groups, 0)
    const int4* cpass64;          // FP64 passes (fewer groups per pass: register budget)
    int npass64;
    const int* vgcol;             // first column of each virtual group (multiple of 32)
    const int* vgsrc;             // offset of its source lanes in src (slots x 32)
    const unsigned char* src;     // per slot and lane: the lane holding the term's value (31: zero)
    const int* ept32;             // combination entries by (pass, output lane), FP32 passes
    const int* eidx32;            //   k << 16 | place of the pair sum in the pass's area
    const float* eg32;            //   coefficient
    const int* ept64;             // the same for the FP64 passes
    const int* eidx64;
    const double* eg64;
};

template <typename T> __device__ __forceinline__ const T* bvals(const BProb& d);
template <> __device__ __forceinline__ const double* bvals<double>(const BProb& d) { return d.vals; }
template <> __device__ __forceinline__ const float* bvals<float>(const BProb& d) { return d.vals32; }
template <typename T> __device__ __forceinline__ const T* bcombg(const BProb& d);
template <> __device__ __forceinline__ const double* bcombg<double>(const BProb& d) { return d.combg; }
template <> __device__ __forceinline__ const float* bcombg<float>(const BProb& d) { return d.combg32; }
template <typename T> __device__ __forceinline__ const T* bdinv(const BProb& d);
template <> __device__ __forceinline__ const double* bdinv<double>(const BProb& d) { return d.dinv; }
template <> __device__ __forceinline__ const float* bdinv<float>(const BProb& d) { return d.dinv32; }

struct sgfem_batch {
    int device = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    std::string err;
    int num_sms = 0;
    bool finalized = false;
    long long launches = 0;
    // host problems
    struct HostProb {
        int n, P, M1, ld;
        std::vector<int> rowptr, col;
        std::vector<double> vals, dinv, b0;
        std::vector<unsigned char> bmask;
        std::vector<int> qtab, combptr, combq;
        std::vector<double> combg;
        double work;
        int nl = 0;          // > 0: dofs are the (nl+1)^2 lattice points, x fastest (sine-transform preconditioner)
        double a0 = 0.0;     // K_0 = a0 * 5-point Laplacian on interior rows
    };
    std::vector<HostProb> hp;
    // device
    std::vector<void*> owned;
    BProb* d_probs = nullptr;
    int* d_bprob = nullptr;
    int* d_vorder = nullptr;      // work-queue order of the virtual blocks (persistent apply)
    int* d_wq = nullptr;          // work-queue counter
    KrylovScalars* d_scal = nullptr;
    double *d_x = nullptr, *d_b = nullptr, *d_r = nullptr, *d_p = nullptr, *d_q = nullptr, *d_part = nullptr;
    double* d_z = nullptr;        // preconditioned residual
    // mixed solve: FP32 inner PCG vectors and the FP64 correction accumulator
    float *d_r32 = nullptr, *d_p32 = nullptr, *d_q32 = nullptr, *d_z32 = nullptr;
    double* d_d64 = nullptr;
    double* d_want = nullptr;     // per-problem squared inner reduction target
    float* d_t = nullptr;         // sine-transform intermediate
    int2* d_dstmap = nullptr;     // (problem, line) per block of the transform passes
    int* d_soff = nullptr;        // per problem: offset of its sine table in d_stab
    float* d_stab = nullptr;      // sine tables of the lattice sizes in the batch
    int ndst = 0;
    int2* d_lat = nullptr;        // per problem: (nl, a0 as float bits); nl = 0: Jacobi
    size_t dst_smem = 0;
    long long total = 0;          // sum of n * ld
    int blocks = 0, wpb = 4, qt = 4, ldmax = 0, m1max = 0, qnmax = 0;
    int wpb32 = 4, qt32 = 8;      // launch shape of the FP32 apply (mixed solve)
    int pf32 = 0;                 // bit 0: the FP32 apply prefetches the next nonzero into registers;
                                  // bit 1: persistent grid over the work queue;
                                  // bit 2: column-slot form (k_bapply_cols)
    int pf64 = 0, wpb64c = 4;     // FP64 apply: 4 = column-slot form with wpb64c warps per block
    bool cols_ok = false;         // every problem has M + 1 <= 31 (the column-slot form applies)
    std::string tuning;
    std::vector<KrylovScalars> h_scal;
    double rtol = 0.0;            // of the last solve
    std::vector<int> h_iters;     // per problem, last solve: PCG iterations (all refinement steps)
    std::vector<double> h_relres; //   and the final ||b - A x|| / ||b|| (FP64)
};

namespace {

constexpr int BT = 256;  // threads of the vector kernels

int bfail(sgfem_batch* b, int code, const std::string& msg) {
    b->err = msg;
    return code;
}
#define BCUDA(b, call)                                                                  \
    do {                                                                                \
        cudaError_t e_ = (call);                                                        \
        if (e_ != cudaSuccess) return bfail(b, SGFEM_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)
#define BLAUNCHED(b)                                                                    \
    do {                                                                                \
        (b)->launches++;                                                                \
        cudaError_t e_ = cudaGetLastError();                                            \
        if (e_ != cudaSuccess) return bfail(b, SGFEM_ERR_CUDA, std::string("launch: ") + cudaGetErrorString(e_)); \
    } while (0)

__device__ __forceinline__ void block_sum_store(double v, double* out) {
    __shared__ double red[32];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += red[w];
        *out = s;
    }
}

// Y = S X for every problem, p'q partials per block.  PF: the next nonzero's X row
// (up to 32 columns per lane, ld <= 1024) and values are loaded into registers
// while the current nonzero's pair FMAs run
constexpr int BPC = 32;  // X columns per lane held for the prefetch
constexpr int BPV = 8;   // KLE values per lane held for the prefetch (M + 1 <= 256)

//
// Work items are the virtual blocks of the block map (problem bprob[v], local index
// v - blk0, partial in partials[v]).  wq == nullptr: one item per launched block
// (v = blockIdx.x).  Otherwise a persistent grid of resident blocks takes items from
// the queue counter *wq (zero at launch) in the order vorder (descending cost) until
// all nvb are taken; the partials land where the plain launch puts them, so the
// per-problem sums stay fixed-order.
template <typename T, int QT, bool PF = false>
__global__ void k_bapply(const BProb* __restrict__ probs, const int* __restrict__ bprob, const T* __restrict__ X,
                         T* __restrict__ Y, double* __restrict__ partials, const KrylovScalars* __restrict__ scal,
                         int per_warp, const int* __restrict__ vorder, int* __restrict__ wq, int nvb) {
    __shared__ int s_item;
    extern __shared__ __align__(16) unsigned char bsm_raw[];
    T* bsm = reinterpret_cast<T*>(bsm_raw);
    const int wpb = blockDim.x >> 5;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int round = 0;; ++round) {
    int vb;
    if (wq) {
        __syncthreads();  // the previous item is finished by every warp (shared area, s_item)
        if (threadIdx.x == 0) {
            const int k = atomicAdd(wq, 1);
            s_item = k < nvb ? vorder[k] : -1;
        }
        __syncthreads();
        vb = s_item;
        if (vb < 0) break;
    } else {
        if (round > 0) break;
        vb = blockIdx.x;
    }
    const int pi = bprob[vb];
    const BProb& d = probs[pi];
    const T* vals = bvals<T>(d);
    const T* combg = bcombg<T>(d);
    if (scal && scal[pi].done) {
        if (threadIdx.x == 0 && partials) partials[vb] = 0.0;
        continue;
    }
    T* su = bsm + (size_t)warp * per_warp;
    T* sc = su + d.ld;
    T* sacc = sc + d.M1 + 1;
    if (lane == 0) sc[d.M1] = T(0);
    const T* Xp = X + d.voff;
    T* Yp = Y + d.voff;
    double dot = 0.0;
    const int lb = vb - d.blk0;
    for (int row = lb * wpb + warp; row < d.n; row += d.nblk * wpb) {
        T* yrow = Yp + (size_t)row * d.ld;
        if (d.bmask[row]) {
            for (int c = lane; c < d.ld; c += 32) yrow[c] = T(0);
            continue;
        }
        const int nz0 = d.rowptr[row], nz1 = d.rowptr[row + 1];
        for (int base = 0; base < d.Qn; base += QT * 32) {
            // the pass's pairs are ordered by column: only columns [c0, c1) of each X row
            // are staged (su[c - c0]); padding lanes read su[0] with a zero value
            const int c0 = d.qtab[base] & 0xffff;
            const int c1 = (d.qtab[min(base + QT * 32, d.Qn) - 1] & 0xffff) + 1;
            const int nc = c1 - c0;
            int om[QT], on[QT];
            T acc[QT];
#pragma unroll
            for (int t = 0; t < QT; ++t) {
                const int q = base + t * 32 + lane;
                if (q < d.Qn) {
                    const int e = d.qtab[q];
                    om[t] = e >> 16;
                    on[t] = (e & 0xffff) - c0;
                } else {
                    om[t] = d.M1;
                    on[t] = 0;
                }
                acc[t] = T(0);
            }
            if constexpr (PF) {
                T xr[BPC], vr[BPV];
                auto fetch = [&](int nz) {
                    const T* xs = Xp + (size_t)d.col[nz] * d.ld + c0;
#pragma unroll
                    for (int u = 0; u < BPC; ++u) {
                        if (32 * u >= nc) break;
                        const int c = lane + 32 * u;
                        xr[u] = c < nc ? __ldg(xs + c) : T(0);
                    }
#pragma unroll
                    for (int u = 0; u < BPV; ++u) {
                        const int m = lane + 32 * u;
                        vr[u] = m < d.M1 ? vals[(size_t)nz * d.M1 + m] : T(0);
                    }
                };
                if (nz0 < nz1) fetch(nz0);
                for (int nz = nz0; nz < nz1; ++nz) {
                    __syncwarp();  // the previous nonzero's FMAs have read su and sc
#pragma unroll
                    for (int u = 0; u < BPC; ++u) {
                        if (32 * u >= nc) break;
                        if (lane + 32 * u < nc) su[lane + 32 * u] = xr[u];
                    }
#pragma unroll
                    for (int u = 0; u < BPV; ++u)
                        if (lane + 32 * u < d.M1) sc[lane + 32 * u] = vr[u];
                    __syncwarp();
                    if (nz + 1 < nz1) fetch(nz + 1);
#pragma unroll
                    for (int t = 0; t < QT; ++t) acc[t] = fma(sc[om[t]], su[on[t]], acc[t]);
                }
                __syncwarp();
            } else {
                for (int nz = nz0; nz < nz1; ++nz) {
                    const int j = d.col[nz];
                    const T* xs = Xp + (size_t)j * d.ld + c0;
                    for (int c = lane; c < nc; c += 32) su[c] = __ldg(xs + c);
                    for (int m = lane; m < d.M1; m += 32) sc[m] = vals[(size_t)nz * d.M1 + m];
                    __syncwarp();
#pragma unroll
                    for (int t = 0; t < QT; ++t) acc[t] = fma(sc[om[t]], su[on[t]], acc[t]);
                    __syncwarp();
                }
            }
#pragma unroll
            for (int t = 0; t < QT; ++t) {
                const int q = base + t * 32 + lane;
                if (q < d.Qn) sacc[q] = acc[t];
            }
        }
        __syncwarp();
        const T* xrow = Xp + (size_t)row * d.ld;
        T rowdot = T(0);  // per-row products in the working precision, rows summed in FP64
        for (int mu = lane; mu < d.ld; mu += 32) {
            T y = T(0);
            if (mu < d.P)  // the first entry is the mode's K_0 pair with g = 1
                for (int e = d.combptr[mu]; e < d.combptr[mu + 1]; ++e) y = fma(combg[e], sacc[d.combq[e]], y);
            yrow[mu] = y;
            rowdot = fma(xrow[mu], y, rowdot);
        }
        dot += (double)rowdot;
        __syncwarp();
    }
    if (partials) {
        __shared__ double red[32];
        for (int o = 16; o > 0; o >>= 1) dot += __shfl_down_sync(0xffffffffu, dot, o);
        if (lane == 0) red[warp] = dot;
        __syncthreads();
        if (threadIdx.x == 0) {
            double s = 0.0;
            for (int w = 0; w < wpb; ++w) s += red[w];
            partials[vb] = s;
        }
        __syncthreads();  // red is free before the next item
    }
    }
}

// ---- column-slot form of the apply: the same Y = S X, scheduled by columns.
// Lane L of a virtual group owns column vgcol + L and keeps NA pair sums
// F[(m, c)] = sum_j K_m[i, j] X[j, c] in registers, one per slot; the M + 1 values of
// a nonzero sit one per lane (lane m holds K_m[i, j], lanes >= M + 1 hold 0) and each
// slot takes its term's value from the lane named by the schedule (__shfl_sync), so
// a lane whose column couples to few terms and one coupled to all of them share the
// instruction stream without a shared-memory gather per pair.  A pass holds GP groups
// of one kind; X[j, c] is read once per group and nonzero (coalesced; a chunk's X
// loads are issued before its FMAs).  After each pass its pair sums go to the warp's
// shared area and every lane adds the pass's entries of its own output columns (the
// K_0 pair with g = 1, then the G entries, as in k_bapply) to the warp's output row.
// kinds: slots per lane 1, 2, 4, 8, 16; groups per pass keep the pair sums of a pass at
// <= 16 per lane, and the pass's X values of a chunk of nonzeros (groups x 4) within
// the 128-register budget
__host__ __device__ constexpr int cols_na(int kind) { return kind == 0 ? 1 : kind == 1 ? 2 : kind == 2 ? 4 : kind == 3 ? 8 : 16; }
__host__ __device__ constexpr int cols_gp(int kind, int es) {
    return es == 4 ? (kind <= 1 ? 8 : kind == 2 ? 4 : kind == 3 ? 2 : 1) : (kind <= 2 ? 4 : kind == 3 ? 2 : 1);
}

template <typename T, int NA, int GP>
__device__ __forceinline__ void cols_pass(const BProb& d, const T* __restrict__ Xp, const T* __restrict__ vals,
                                          int nz0, int nz1, int vg0, int ng, T* __restrict__ sacc, int lane) {
    // groups g >= ng of a short pass read lane 31 (zero) in every slot; columns past the
    // row are clamped into it (their slots read zero too), so the loops below have no
    // per-group or per-nonzero branch
    int src[GP][NA];
    int cbc[GP];
    T acc[GP][NA];
#pragma unroll
    for (int g = 0; g < GP; ++g) {
        const bool on = g < ng;
        const int vg = vg0 + (on ? g : 0);
        cbc[g] = min(d.vgcol[vg] + lane, d.ld - 1);
        const unsigned char* sp = d.src + d.vgsrc[vg] + lane;
#pragma unroll
        for (int s = 0; s < NA; ++s) {
            src[g][s] = on ? (int)sp[32 * s] : 31;
            acc[g][s] = T(0);
        }
    }
    // the row's nonzeros in chunks of CH = 4: lane t holds the column of nonzero base + t and
    // lane m the K_m value of each (zero past the row's end, whose column reads row 0),
    // so the X loads of a chunk depend on no other load; they are issued two nonzeros
    // ahead of their FMAs
    constexpr int CH = 4;
    for (int base = nz0; base < nz1; base += CH) {
        const int cnt = min(CH, nz1 - base);
        const int jl = lane < cnt ? __ldg(d.col + base + lane) : 0;
        T kr[CH];
#pragma unroll
        for (int t = 0; t < CH; ++t) kr[t] = (t < cnt && lane < d.M1) ? vals[(size_t)(base + t) * d.M1 + lane] : T(0);
        T ux[CH][GP];
#pragma unroll
        for (int t = 0; t < 2; ++t) {
            const T* xr = Xp + (size_t)__shfl_sync(0xffffffffu, jl, t) * d.ld;
#pragma unroll
            for (int g = 0; g < GP; ++g) ux[t][g] = __ldg(xr + cbc[g]);
        }
#pragma unroll
        for (int t = 0; t < CH; ++t) {
            if (t + 2 < CH) {
                const T* xr = Xp + (size_t)__shfl_sync(0xffffffffu, jl, t + 2) * d.ld;
#pragma unroll
                for (int g = 0; g < GP; ++g) ux[t + 2][g] = __ldg(xr + cbc[g]);
            }
#pragma unroll
            for (int g = 0; g < GP; ++g)
#pragma unroll
                for (int s = 0; s < NA; ++s)
                    acc[g][s] = fma(__shfl_sync(0xffffffffu, kr[t], src[g][s]), ux[t][g], acc[g][s]);
        }
    }
    // the pass's pair sums to the warp's area: group g, slot s, lane L at (g NA + s) 32 + L
#pragma unroll
    for (int g = 0; g < GP; ++g) {
        if (g < ng) {
#pragma unroll
            for (int s = 0; s < NA; ++s) sacc[(g * NA + s) * 32 + lane] = acc[g][s];
        }
    }
}

// pair sums per lane of one pass: at most 16
template <typename T>
__host__ __device__ constexpr int cols_area() { return 16 * 32; }

// work items as in k_bapply (block map or persistent queue); the warp's shared area is
// the pass area (cols_area) followed by the output row (per_warp - cols_area values);
// after every pass each lane adds the pass's entries of its own output columns
// (32 k + lane) to the row, so no lane writes another lane's outputs
template <typename T>
__global__ void __launch_bounds__(256, 2) k_bapply_cols(const BProb* __restrict__ probs, const int* __restrict__ bprob, const T* __restrict__ X,
                              T* __restrict__ Y, double* __restrict__ partials, const KrylovScalars* __restrict__ scal,
                              int per_warp, const int* __restrict__ vorder, int* __restrict__ wq, int nvb) {
    __shared__ int s_item;
    extern __shared__ __align__(16) unsigned char bsm_raw[];
    T* bsm = reinterpret_cast<T*>(bsm_raw);
    const int wpb = blockDim.x >> 5;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int round = 0;; ++round) {
        int vb;
        if (wq) {
            __syncthreads();
            if (threadIdx.x == 0) {
                const int k = atomicAdd(wq, 1);
                s_item = k < nvb ? vorder[k] : -1;
            }
            __syncthreads();
            vb = s_item;
            if (vb < 0) break;
        } else {
            if (round > 0) break;
            vb = blockIdx.x;
        }
        const int pi = bprob[vb];
        const BProb& d = probs[pi];
        const T* vals = bvals<T>(d);
        if (scal && scal[pi].done) {
            if (threadIdx.x == 0 && partials) partials[vb] = 0.0;
            continue;
        }
        T* sacc = bsm + (size_t)warp * per_warp;
        T* ys = sacc + cols_area<T>();
        constexpr int ES = (int)sizeof(T);
        const int* ept = ES == 4 ? d.ept32 : d.ept64;
        const int* eidx = ES == 4 ? d.eidx32 : d.eidx64;
        const T* eg = ES == 4 ? reinterpret_cast<const T*>(d.eg32) : reinterpret_cast<const T*>(d.eg64);
        const T* Xp = X + d.voff;
        T* Yp = Y + d.voff;
        double dot = 0.0;
        const int lb = vb - d.blk0;
        for (int row = lb * wpb + warp; row < d.n; row += d.nblk * wpb) {
            T* yrow = Yp + (size_t)row * d.ld;
            if (d.bmask[row]) {
                for (int c = lane; c < d.ld; c += 32) yrow[c] = T(0);
                continue;
            }
            const int nz0 = d.rowptr[row], nz1 = d.rowptr[row + 1];
            for (int mu = lane; mu < d.ld; mu += 32) ys[mu] = T(0);
            const int np = ES == 4 ? d.npass : d.npass64;
            const int4* cp = ES == 4 ? d.cpass : d.cpass64;
            for (int p = 0; p < np; ++p) {
                const int4 ps = cp[p];
                // passes of one group take the one-group form (no padding groups)
                switch (2 * ps.x + (ps.z == 1)) {
                    case 0: cols_pass<T, cols_na(0), cols_gp(0, ES)>(d, Xp, vals, nz0, nz1, ps.y, ps.z, sacc, lane); break;
                    case 1: cols_pass<T, cols_na(0), 1>(d, Xp, vals, nz0, nz1, ps.y, 1, sacc, lane); break;
                    case 2: cols_pass<T, cols_na(1), cols_gp(1, ES)>(d, Xp, vals, nz0, nz1, ps.y, ps.z, sacc, lane); break;
                    case 3: cols_pass<T, cols_na(1), 1>(d, Xp, vals, nz0, nz1, ps.y, 1, sacc, lane); break;
                    case 4: cols_pass<T, cols_na(2), cols_gp(2, ES)>(d, Xp, vals, nz0, nz1, ps.y, ps.z, sacc, lane); break;
                    case 5: cols_pass<T, cols_na(2), 1>(d, Xp, vals, nz0, nz1, ps.y, 1, sacc, lane); break;
                    case 6: cols_pass<T, cols_na(3), cols_gp(3, ES)>(d, Xp, vals, nz0, nz1, ps.y, ps.z, sacc, lane); break;
                    case 7: cols_pass<T, cols_na(3), 1>(d, Xp, vals, nz0, nz1, ps.y, 1, sacc, lane); break;
                    case 8: cols_pass<T, cols_na(4), cols_gp(4, ES)>(d, Xp, vals, nz0, nz1, ps.y, ps.z, sacc, lane); break;
                    default: cols_pass<T, cols_na(4), 1>(d, Xp, vals, nz0, nz1, ps.y, 1, sacc, lane); break;
                }
                __syncwarp();  // the pass's sums are in the area
                const int e1 = __ldg(ept + p * 32 + lane + 1);
                for (int e = __ldg(ept + p * 32 + lane); e < e1; ++e) {
                    const int v = __ldg(eidx + e);
                    T* yo = ys + (v >> 16) * 32 + lane;
                    *yo = fma(__ldg(eg + e), sacc[v & 0xffff], *yo);
                }
                __syncwarp();  // the area is read before the next pass writes it
            }
            const T* xrow = Xp + (size_t)row * d.ld;
            T rowdot = T(0);
            for (int mu = lane; mu < d.ld; mu += 32) {
                const T y = ys[mu];
                yrow[mu] = y;
                rowdot = fma(xrow[mu], y, rowdot);
            }
            dot += (double)rowdot;
        }
        if (partials) {
            __shared__ double red[32];
            for (int o = 16; o > 0; o >>= 1) dot += __shfl_down_sync(0xffffffffu, dot, o);
            if (lane == 0) red[warp] = dot;
            __syncthreads();
            if (threadIdx.x == 0) {
                double s = 0.0;
                for (int w = 0; w < wpb; ++w) s += red[w];
                partials[vb] = s;
            }
            __syncthreads();
        }
    }
}

enum BFin { BF_ALPHA = 0, BF_RR = 1, BF_BETA = 2, BF_TOL = 3, BF_NORM = 4 };

// one block per problem: sum its block partials in order, update its scalars
// (BF_TOL: tol2 = rtol2 * sum, rtol2 per problem when want != nullptr; BF_NORM: rr = sum)
__global__ void k_bfin(const BProb* __restrict__ probs, const double* __restrict__ partials,
                       KrylovScalars* __restrict__ scal, int mode, double rtol2, int maxit,
                       const double* __restrict__ want = nullptr) {
    const BProb& d = probs[blockIdx.x];
    KrylovScalars* s = scal + blockIdx.x;
    __shared__ double red[BT];
    double v = 0.0;
    for (int i = threadIdx.x; i < d.nblk; i += BT) v += partials[d.blk0 + i];
    red[threadIdx.x] = v;
    __syncthreads();
    for (int w = BT / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x != 0) return;
    const double sum = red[0];
    if (mode == BF_TOL) {
        s->tol2 = (want ? want[blockIdx.x] : rtol2) * sum;
        s->rr = sum;
        if (sum == 0.0) s->done = 1;
        return;
    }
    if (mode == BF_NORM) {
        s->rr = sum;
        return;
    }
    if (s->done) return;
    if (mode == BF_ALPHA) {
        s->pq = sum;
        if (!isfinite(sum)) { s->status = SGFEM_ERR_NONFINITE; s->done = 1; return; }
        if (!(sum > 0.0)) { s->status = SGFEM_ERR_BREAKDOWN; s->done = 1; return; }
        s->alpha = s->rho / sum;
    } else if (mode == BF_RR) {
        s->rr = sum;
        if (!s->first) s->iters += 1;
        if (!isfinite(sum)) { s->status = SGFEM_ERR_NONFINITE; s->done = 1; return; }
        if (sum <= s->tol2) { s->done = 1; return; }
        if (s->iters >= maxit) { s->status = SGFEM_ERR_MAXIT; s->done = 1; return; }
    } else if (mode == BF_BETA) {
        if (!isfinite(sum)) { s->status = SGFEM_ERR_NONFINITE; s->done = 1; return; }
        if (!(sum > 0.0)) { s->status = SGFEM_ERR_BREAKDOWN; s->done = 1; return; }
        s->beta = s->first ? 0.0 : sum / s->rho;
        s->first = 0;
        s->rho = sum;
    }
}

// element range of block blockIdx.x within its problem's vectors
#define BRANGE                                                                          \
    const int pi = bprob[blockIdx.x];                                                   \
    const BProb& d = probs[pi];                                                         \
    const long long len = (long long)d.n * d.ld;                                        \
    const long long t0 = (long long)(blockIdx.x - d.blk0) * BT + threadIdx.x;          \
    const long long tstep = (long long)d.nblk * BT;

// x += alpha p, r -= alpha q, ||r||^2 partials (TX = double with T = float: the FP32
// PCG's solution accumulates in FP64; partials per thread in T)
template <typename T, typename TX>
__global__ void __launch_bounds__(BT) k_bupdate(const BProb* __restrict__ probs, const int* __restrict__ bprob,
                                                TX* __restrict__ x, const T* __restrict__ p, T* __restrict__ r,
                                                const T* __restrict__ q, const KrylovScalars* __restrict__ scal,
                                                double* __restrict__ partials) {
    BRANGE;
    T acc = T(0);
    if (!scal[pi].done) {
        const T a = (T)scal[pi].alpha;
        const TX ax = (TX)scal[pi].alpha;
        for (long long t = t0; t < len; t += tstep) {
            const long long i = d.voff + t;
            x[i] = fma(ax, (TX)p[i], x[i]);
            const T rn = fma(-a, q[i], r[i]);
            r[i] = rn;
            acc = fma(rn, rn, acc);
        }
    }
    block_sum_store((double)acc, partials + blockIdx.x);
}

// mixed solve: r32 = (float) r, d = 0, partials of ||r32||^2 (problems with done set skip)
__global__ void __launch_bounds__(BT) k_bdemote(const BProb* __restrict__ probs, const int* __restrict__ bprob,
                                                const double* __restrict__ r, float* __restrict__ r32,
                                                double* __restrict__ dx, double* __restrict__ partials) {
    BRANGE;
    float acc = 0.f;
    for (long long t = t0; t < len; t += tstep) {
        const long long i = d.voff + t;
        const float v = (float)r[i];
        r32[i] = v;
        dx[i] = 0.0;
        acc = fmaf(v, v, acc);
    }
    block_sum_store((double)acc, partials + blockIdx.x);
}

// mixed solve: x += d, r = b - q (q = A x from the FP64 apply), partials of ||r||^2
__global__ void __launch_bounds__(BT) k_badd(const BProb* __restrict__ probs, const int* __restrict__ bprob,
                                             double* __restrict__ x, const double* __restrict__ dx) {
    BRANGE;
    for (long long t = t0; t < len; t += tstep) x[d.voff + t] += dx[d.voff + t];
}
__global__ void __launch_bounds__(BT) k_bresid(const BProb* __restrict__ probs, const int* __restrict__ bprob,
                                               const double* __restrict__ b, const double* __restrict__ q,
                                               double* __restrict__ r, double* __restrict__ partials) {
    BRANGE;
    double acc = 0.0;
    for (long long t = t0; t < len; t += tstep) {
        const long long i = d.voff + t;
        const double rv = b[i] - q[i];
        r[i] = rv;
        acc = fma(rv, rv, acc);
    }
    block_sum_store(acc, partials + blockIdx.x);
}

// mode 0: partials of r' D^-1 r ; mode 1: p = D^-1 r + beta p ; mode 2: partials of b'b
template <typename T>
__global__ void __launch_bounds__(BT) k_bjacobi(const BProb* __restrict__ probs, const int* __restrict__ bprob,
                                                const T* __restrict__ r, T* __restrict__ p,
                                                const KrylovScalars* __restrict__ scal, double* __restrict__ partials,
                                                int mode) {
    BRANGE;
    T acc = T(0);
    const T* dinv = bdinv<T>(d);
    if (mode == 2 || !scal[pi].done) {
        const T beta = (mode == 1) ? (T)scal[pi].beta : T(0);
        for (long long t = t0; t < len; t += tstep) {
            const long long i = d.voff + t;
            const T rv = r[i];
            if (mode == 2) {
                acc = fma(rv, rv, acc);
                continue;
            }
            const T z = dinv[t / d.ld] * rv;
            if (mode == 0)
                acc = fma(rv, z, acc);
            else
                p[i] = fma(beta, p[i], z);
        }
    }
    if (mode != 1) block_sum_store((double)acc, partials + blockIdx.x);
}

// b = e_1 (x) b0 (Dirichlet rows zero) in the device layout; x = 0
__global__ void k_brhs(const double* __restrict__ b0, long long off_b0, double* __restrict__ b, double* __restrict__ x,
                       long long voff, int n, int ld, const unsigned char* __restrict__ bmask) {
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < (long long)n * ld;
         t += (long long)gridDim.x * blockDim.x) {
        const int row = (int)(t / ld), c = (int)(t % ld);
        b[voff + t] = (c == 0 && !bmask[row]) ? b0[off_b0 + row] : 0.0;
        x[voff + t] = 0.0;
    }
}

// device layout (n x ld, row-major) -> caller layout (n x P column-major)
__global__ void k_bout(const double* __restrict__ x, long long voff, int n, int ld, int P, double* __restrict__ out,
                       long long ooff) {
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < (long long)n * P;
         t += (long long)gridDim.x * blockDim.x) {
        const int c = (int)(t / n), row = (int)(t % n);
        out[ooff + t] = x[voff + (long long)row * ld + c];
    }
}

// z = D^-1 r on the problems without a lattice (Jacobi), Dirichlet rows zero
template <typename T>
__global__ void __launch_bounds__(BT) k_bjz(const BProb* __restrict__ probs, const int* __restrict__ bprob,
                                            const int2* __restrict__ lat, const T* __restrict__ r,
                                            T* __restrict__ z, const KrylovScalars* __restrict__ scal) {
    BRANGE;
    if (lat[pi].x > 0 || scal[pi].done) return;
    const T* dinv = bdinv<T>(d);
    for (long long t = t0; t < len; t += tstep) z[d.voff + t] = dinv[t / d.ld] * r[d.voff + t];
}

// partials of r'z per block of each problem
template <typename T>
__global__ void __launch_bounds__(BT) k_brz(const BProb* __restrict__ probs, const int* __restrict__ bprob,
                                            const T* __restrict__ r, const T* __restrict__ z,
                                            const KrylovScalars* __restrict__ scal, double* __restrict__ partials) {
    BRANGE;
    T acc = T(0);
    if (!scal[pi].done)
        for (long long t = t0; t < len; t += tstep) acc = fma(r[d.voff + t], z[d.voff + t], acc);
    block_sum_store((double)acc, partials + blockIdx.x);
}

// p = z + beta p
template <typename T>
__global__ void __launch_bounds__(BT) k_bpz(const BProb* __restrict__ probs, const int* __restrict__ bprob,
                                            const T* __restrict__ z, T* __restrict__ p,
                                            const KrylovScalars* __restrict__ scal) {
    BRANGE;
    if (scal[pi].done) return;
    const T beta = (T)scal[pi].beta;
    for (long long t = t0; t < len; t += tstep) p[d.voff + t] = fma(beta, p[d.voff + t], z[d.voff + t]);
}

// Mean-based preconditioner of a lattice problem, z = (a0 L)^-1 r on interior rows
// (L the 5-point Laplacian of the (nl+1)^2 lattice), by the sine transform
// S_ik = sin(pi i k / nl), i, k = 1..N = nl-1 (S^2 = (nl/2) I), applied as a dense
// matrix product along every lattice line: pass 0 (x): t = S r per line j;
// pass 1 (y): t = S (D .* (S t)) per column, D = (2/nl)^2 / (a0 (lam_kx + lam_ky)),
// lam_k = 4 sin^2(pi k / (2 nl)); pass 2 (x): z = S t per line.  FP32 arithmetic.
// Each product is split by the parity of the output: S_{i,nl-k} = S_ik for odd i and
// -S_ik for even i, so with u_k = x_k + x_{nl-k}, v_k = x_k - x_{nl-k} (k <= H =
// (nl-1)/2, and the middle point x_{nl/2} for even nl, which only odd i see)
//   y_i (odd i)  = sum_k S_ik u_k (+ sin(pi i / 2) x_{nl/2}),
//   y_i (even i) = sum_k S_ik v_k,
// two products of half the size: half the FMAs of S x.  In the tile the pair
// (k, nl - k) becomes (u_k, v_k) in place, so rows 0..HU-1 hold u (and the middle
// point) and rows HU..N-1 hold v_H..v_1.  The tables (built at finalize, transposed
// so that row r holds the coefficients of consecutive outputs, padded with zeros to
// 16 outputs) are TO (HU x NOP, odd outputs) and TE (H x NEP, even outputs).
// One block per (problem, line): the tables are staged in shared memory once, then
// the line's columns go in chunks of cw; each warp computes 16 outputs x 64 columns
// (2 columns per lane: one float2 tile load and four broadcast float4 table loads
// per 32 packed FMAs); cw = 64 * (8 / output blocks) keeps the 8 warps busy.
constexpr int DST_WARPS = 8;

struct DstShape {
    int N, H, HU, no, ne, NOP, NEP, nro, nre, cpw, cw, tab;  // tab: table floats (TO, TE, LAM)
};
__host__ __device__ inline DstShape dst_shape(int nl) {
    DstShape q;
    q.N = nl - 1;
    q.H = (nl - 1) / 2;
    q.HU = q.H + (nl % 2 == 0 ? 1 : 0);
    q.no = (q.N + 1) / 2;
    q.ne = q.N / 2;
    q.NOP = (q.no + 15) & ~15;
    q.NEP = q.ne > 0 ? (q.ne + 15) & ~15 : 0;
    q.nro = q.NOP / 16;
    q.nre = q.NEP / 16;
    q.cpw = DST_WARPS / (q.nro + q.nre);
    q.cw = 64 * q.cpw;
    q.tab = q.HU * q.NOP + q.H * q.NEP + ((q.N + 15) & ~15);
    return q;
}

// (x_k, x_{nl-k}) -> (u_k, v_k) for k = 1..H over the whole N x cw tile
__device__ __forceinline__ void dst_butterfly(float* tile, int nl, int H, int cw) {
    for (int i = threadIdx.x; i < H * (cw / 4); i += blockDim.x) {
        const int k = 1 + i / (cw / 4), c = 4 * (i % (cw / 4));
        float4* pa = reinterpret_cast<float4*>(tile + (k - 1) * cw + c);
        float4* pb = reinterpret_cast<float4*>(tile + (nl - k - 1) * cw + c);
        const float4 a = *pa, b = *pb;
        *pa = make_float4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w);
        *pb = make_float4(a.x - b.x, a.y - b.y, a.z - b.z, a.w - b.w);
    }
}

// acc[i] = sum_k tab[k * tstride + i] * tile[k * cw + col .. + 1] for 16 outputs i
__device__ __forceinline__ void dst_unit(float2 (&acc)[16], const float* __restrict__ tab, int tstride,
                                         const float* __restrict__ tr, int cw, int kin) {
#pragma unroll
    for (int i = 0; i < 16; ++i) acc[i] = make_float2(0.f, 0.f);
#pragma unroll 2
    for (int k = 0; k < kin; ++k) {
        const float2 x = *reinterpret_cast<const float2*>(tr + k * cw);
        const float4* s4 = reinterpret_cast<const float4*>(tab + k * tstride);
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const float4 sv = s4[j];
            acc[4 * j + 0] = __ffma2_rn(make_float2(sv.x, sv.x), x, acc[4 * j + 0]);
            acc[4 * j + 1] = __ffma2_rn(make_float2(sv.y, sv.y), x, acc[4 * j + 1]);
            acc[4 * j + 2] = __ffma2_rn(make_float2(sv.z, sv.z), x, acc[4 * j + 2]);
            acc[4 * j + 3] = __ffma2_rn(make_float2(sv.w, sv.w), x, acc[4 * j + 3]);
        }
    }
}

template <typename T>
__global__ void __launch_bounds__(DST_WARPS * 32, 2) k_bdst(const BProb* __restrict__ probs, const int2* __restrict__ map,
                                                            const int2* __restrict__ lat, const int* __restrict__ soff,
                                                            const float* __restrict__ stab, int pass,
                                                            const T* __restrict__ r, float* __restrict__ t,
                                                            T* __restrict__ z, const KrylovScalars* __restrict__ scal) {
    const int2 e = map[blockIdx.x];
    const int pi = e.x, line = e.y;
    if (scal[pi].done) return;
    const BProb& d = probs[pi];
    const int nl = lat[pi].x;
    const DstShape q = dst_shape(nl);
    const int N = q.N, cw = q.cw;
    const float a0 = __int_as_float(lat[pi].y);
    extern __shared__ __align__(16) float dsm[];
    float* TO = dsm;                    // HU x NOP
    float* TE = TO + q.HU * q.NOP;      // H x NEP
    const float* LAM = TE + q.H * q.NEP; // lam_k = 4 sin^2(pi k / (2 nl)), k = 1..N
    float* tile = dsm + q.tab;          // N x cw
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    {
        const float4* src = reinterpret_cast<const float4*>(stab + soff[pi]);
        float4* dst = reinterpret_cast<float4*>(dsm);
        for (int i = threadIdx.x; i < q.tab / 4; i += blockDim.x) dst[i] = __ldg(src + i);
    }
    const int stride = nl + 1;
    auto row_of = [&](int k) { return (pass == 1) ? k * stride + line : line * stride + k; };  // k = 1..N
    // this warp's unit: output block rb (odd outputs for rb < nro, even after), columns 64 cc + 2 lane
    const int nrb = q.nro + q.nre;
    const int rb = warp % nrb, cc = warp / nrb;
    const bool busy = warp < nrb * q.cpw;
    const bool odd = rb < q.nro;
    const int ob = odd ? rb : rb - q.nro;                    // block within its parity
    const float* tab = odd ? TO + 16 * ob : TE + 16 * ob;    // row r at tab + r * tstride
    const int tstride = odd ? q.NOP : q.NEP;
    const int kin = odd ? q.HU : q.H;                        // inner length
    const int roff = odd ? 0 : q.HU;                         // first tile row of the inner range
    const int nout = odd ? q.no : q.ne;
    const int col = 64 * cc + 2 * lane;
    float2 acc[16];
    const float* tr = tile + roff * cw + col;
    for (int c0 = 0; c0 < d.ld; c0 += cw) {
        __syncthreads();  // tables staged / the previous chunk's tile read
        const int cn = min(cw, d.ld - c0);  // a multiple of 4
        for (int i = threadIdx.x; i < N * (cw / 4); i += blockDim.x) {
            const int k = i / (cw / 4), c = 4 * (i - k * (cw / 4));
            float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
            if (c < cn) {
                const long long idx = d.voff + (long long)row_of(k + 1) * d.ld + c0 + c;
                if (pass == 0) {
                    if constexpr (sizeof(T) == 8) {
                        const double2 v0 = *reinterpret_cast<const double2*>(r + idx);
                        const double2 v1 = *reinterpret_cast<const double2*>(r + idx + 2);
                        v = make_float4((float)v0.x, (float)v0.y, (float)v1.x, (float)v1.y);
                    } else {
                        v = *reinterpret_cast<const float4*>(r + idx);
                    }
                } else {
                    v = *reinterpret_cast<const float4*>(t + idx);
                }
            }
            *reinterpret_cast<float4*>(tile + k * cw + c) = v;
        }
        __syncthreads();
        dst_butterfly(tile, nl, q.H, cw);
        __syncthreads();
        if (busy) dst_unit(acc, tab, tstride, tr, cw, kin);
        if (pass == 1) {
            // scale output i (tile row i - 1) by D(kx = line, ky = i), split again, transform again
            __syncthreads();  // every warp has read the tile
            if (busy) {
                const float lx = LAM[line - 1];
                const float nrm = 4.f / ((float)nl * (float)nl);
#pragma unroll
                for (int i = 0; i < 16; ++i) {
                    const int j = 16 * ob + i;
                    if (j < nout) {
                        const int orow = odd ? 2 * j : 2 * j + 1;
                        const float f = nrm / (a0 * (lx + LAM[orow]));
                        *reinterpret_cast<float2*>(tile + orow * cw + col) = make_float2(acc[i].x * f, acc[i].y * f);
                    }
                }
            }
            __syncthreads();
            dst_butterfly(tile, nl, q.H, cw);
            __syncthreads();
            if (busy) dst_unit(acc, tab, tstride, tr, cw, kin);
        }
        if (busy && col < cn) {
#pragma unroll
            for (int i = 0; i < 16; ++i) {
                const int j = 16 * ob + i;
                if (j < nout) {
                    const int orow = odd ? 2 * j : 2 * j + 1;
                    const long long idx = d.voff + (long long)row_of(orow + 1) * d.ld + c0 + col;
                    if (pass == 2) {
                        z[idx] = (T)acc[i].x;
                        z[idx + 1] = (T)acc[i].y;
                    } else {
                        *reinterpret_cast<float2*>(t + idx) = acc[i];
                    }
                }
            }
        }
    }
}

template <typename Tv>
int bupload(sgfem_batch* b, const std::vector<Tv>& v, Tv** dst) {
    void* p = nullptr;
    BCUDA(b, cudaMalloc(&p, std::max<size_t>(v.size(), 1) * sizeof(Tv)));
    b->owned.push_back(p);
    if (!v.empty()) BCUDA(b, cudaMemcpy(p, v.data(), v.size() * sizeof(Tv), cudaMemcpyHostToDevice));
    *dst = (Tv*)p;
    return SGFEM_OK;
}

int balloc(sgfem_batch* b, size_t bytes, void** dst) {
    BCUDA(b, cudaMalloc(dst, std::max<size_t>(bytes, 8)));
    b->owned.push_back(*dst);
    return SGFEM_OK;
}

template <typename T = double>
size_t apply_smem(const sgfem_batch* b, int wpb, int pf = 0) {
    if (pf & 4) return (size_t)(cols_area<T>() + ((b->ldmax + 3) & ~3)) * sizeof(T) * wpb;
    const size_t per_warp = ((size_t)b->ldmax + b->m1max + 1 + b->qnmax + 3) & ~(size_t)3;
    return per_warp * sizeof(T) * wpb;
}

// pf bit 0: the prefetching variant (FP32, 16 or 32 pairs per lane); bit 1: persistent
// grid over the work queue (resident blocks only, queue counter reset before the launch);
// bit 2: the column-slot form (qt unused)
template <typename T>
int launch_apply(sgfem_batch* b, int wpb, int qt, const T* X, T* Y, double* partials, const KrylovScalars* scal,
                 int pf = 0) {
    const int per_warp = (pf & 4) ? cols_area<T>() + ((b->ldmax + 3) & ~3)
                                  : (int)(((size_t)b->ldmax + b->m1max + 1 + b->qnmax + 3) & ~(size_t)3);
    const size_t smem = apply_smem<T>(b, wpb, pf);
    using KF = void (*)(const BProb*, const int*, const T*, T*, double*, const KrylovScalars*, int, const int*, int*, int);
    KF kf;
    if (pf & 4) kf = k_bapply_cols<T>;
    else if (pf & 1) kf = qt == 16 ? k_bapply<T, 16, true> : k_bapply<T, 32, true>;
    else kf = qt == 4 ? k_bapply<T, 4> : qt == 8 ? k_bapply<T, 8> : qt == 16 ? k_bapply<T, 16> : k_bapply<T, 32>;
    int grid = b->blocks;
    int* wq = nullptr;
    if (pf & 2) {
        int per_sm = 0;
        BCUDA(b, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kf, wpb * 32, smem));
        grid = std::min(b->blocks, std::max(1, per_sm) * b->num_sms);
        BCUDA(b, cudaMemsetAsync(b->d_wq, 0, sizeof(int), b->stream));
        wq = b->d_wq;
    }
    kf<<<grid, wpb * 32, smem, b->stream>>>(b->d_probs, b->d_bprob, X, Y, partials, scal, per_warp, b->d_vorder, wq,
                                            b->blocks);
    BLAUNCHED(b);
    return SGFEM_OK;
}

// the apply kernel of a form and its shared-memory opt-in (above the 48 KB default)
template <typename T>
const void* apply_kernel(int pf, int qt) {
    if (pf & 4) return (const void*)k_bapply_cols<T>;
    if (pf & 1) return qt == 16 ? (const void*)k_bapply<T, 16, true> : (const void*)k_bapply<T, 32, true>;
    return qt == 4 ? (const void*)k_bapply<T, 4> : qt == 8 ? (const void*)k_bapply<T, 8>
         : qt == 16 ? (const void*)k_bapply<T, 16> : (const void*)k_bapply<T, 32>;
}
template <typename T>
cudaError_t set_apply_smem(int pf, int qt, size_t smem) {
    if (smem <= 48 * 1024) return cudaSuccess;
    return cudaFuncSetAttribute(apply_kernel<T>(pf, qt), cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
}

// FP64 apply in the chosen form (pair passes or column slots)
int apply64(sgfem_batch* b, const double* X, double* Y, double* partials, const KrylovScalars* scal) {
    if (b->pf64 & 4) return launch_apply<double>(b, b->wpb64c, 0, X, Y, partials, scal, b->pf64);
    return launch_apply<double>(b, b->wpb, b->qt, X, Y, partials, scal);
}

// the block map and the work-queue order (virtual blocks by descending rows x pairs each) to the device
int upload_map(sgfem_batch* b, const std::vector<BProb>& probs, const std::vector<int>& bprob) {
    std::vector<int> order(bprob.size());
    std::iota(order.begin(), order.end(), 0);
    auto cost = [&](int v) { return b->hp[bprob[v]].work / probs[bprob[v]].nblk; };
    std::stable_sort(order.begin(), order.end(), [&](int u, int v) { return cost(u) > cost(v); });
    BCUDA(b, cudaMemcpy(b->d_probs, probs.data(), probs.size() * sizeof(BProb), cudaMemcpyHostToDevice));
    BCUDA(b, cudaMemcpy(b->d_bprob, bprob.data(), bprob.size() * sizeof(int), cudaMemcpyHostToDevice));
    BCUDA(b, cudaMemcpy(b->d_vorder, order.data(), order.size() * sizeof(int), cudaMemcpyHostToDevice));
    return SGFEM_OK;
}

// block ranges proportional to the problems' work for a given total
int build_map(sgfem_batch* b, int total_blocks, std::vector<BProb>& probs, std::vector<int>& bprob) {
    const int B = (int)b->hp.size();
    double wsum = 0.0;
    for (auto& h : b->hp) wsum += h.work;
    std::vector<int> nb(B);
    int used = 0;
    for (int i = 0; i < B; ++i) {
        nb[i] = std::max(1, (int)std::lround(total_blocks * b->hp[i].work / wsum));
        // no more blocks than rows (apply) or useful vector chunks
        nb[i] = std::min(nb[i], std::max(1, b->hp[i].n));
        used += nb[i];
    }
    bprob.assign(used, 0);
    int at = 0;
    for (int i = 0; i < B; ++i) {
        probs[i].blk0 = at;
        probs[i].nblk = nb[i];
        for (int k = 0; k < nb[i]; ++k) bprob[at + k] = i;
        at += nb[i];
    }
    b->blocks = used;
    return SGFEM_OK;
}

// The split sine tables of one lattice size, appended to out (k_bdst's layout):
// TO[r][j] (odd output i = 2j + 1): sin(pi i (r + 1) / nl) for r < H, sin(pi i / 2) for
// the middle point (r = H, even nl); TE[r][j] (even output i = 2j + 2): sin(pi i (H - r)
// / nl); LAM[k - 1] = 4 sin^2(pi k / (2 nl)), the 1-D Laplacian eigenvalues of pass 1's
// scaling.  Columns past the last output and LAM past N are zero.
void dst_tables(int nl, std::vector<float>& out) {
    const DstShape q = dst_shape(nl);
    for (int r = 0; r < q.HU; ++r)
        for (int j = 0; j < q.NOP; ++j) {
            const int io = 2 * j + 1;
            const int k = r < q.H ? r + 1 : 0;
            double v = 0.0;
            if (j < q.no) v = r < q.H ? std::sin(M_PI * (double)((io * k) % (2 * nl)) / nl) : std::sin(M_PI * 0.5 * io);
            out.push_back((float)v);
        }
    for (int r = 0; r < q.H; ++r)
        for (int j = 0; j < q.NEP; ++j) {
            const int ie = 2 * j + 2, k = q.H - r;
            out.push_back(j < q.ne ? (float)std::sin(M_PI * (double)((ie * k) % (2 * nl)) / nl) : 0.f);
        }
    for (int k = 1; k <= ((q.N + 15) & ~15); ++k) {
        const double sk = std::sin(M_PI * k / (2.0 * nl));
        out.push_back(k <= q.N ? (float)(4.0 * sk * sk) : 0.f);
    }
}

// ---- schedule of the column-slot apply for one problem.  Column block b holds columns
// 32 b + L; lane L's terms are the m with (m, column) in the pair list, in increasing m.
// The block's longest list is cut into virtual groups of 16, 8, 4, 2 or 1 slots (a
// remainder of 3 or 7 is rounded up to 4 or 8: one idle slot costs less than another
// group); lanes with fewer terms, and columns >= P, read lane 31, which holds zero.
// Passes take up to GP groups of one kind; the pair sums of the groups follow one
// another in the warp's area in pass order.
struct ColSched {
    std::vector<int4> pass, pass64;
    std::vector<int> vgcol, vgsrc;
    std::vector<unsigned char> src;
    // combination entries per precision, grouped by (pass, lane of the output column):
    // ept[p * 32 + L] .. ept[p * 32 + L + 1] index eidx (k << 16 | place in the pass's
    // area; output column 32 k + L) and eg (coefficient)
    std::vector<int> ept32, eidx32, ept64, eidx64;
    std::vector<double> eg32, eg64;
};

void build_cols(const sgfem_batch::HostProb& h, ColSched& cs) {
    const int P = h.P, M1 = h.M1;
    std::vector<std::vector<int>> terms(P);
    for (int e : h.qtab) terms[e & 0xffff].push_back(e >> 16);
    for (auto& t : terms) std::sort(t.begin(), t.end());
    struct VG { int kind, col, first; };  // first: index of the lane's first term in this group
    std::vector<VG> vgs;
    for (int b0 = 0; b0 < P; b0 += 32) {
        int amax = 0;
        for (int c = b0; c < std::min(P, b0 + 32); ++c) amax = std::max(amax, (int)terms[c].size());
        int first = 0, r = amax;
        while (r > 0) {
            int na = r >= 16 ? 16 : r >= 8 ? (r == 15 ? 16 : 8) : r >= 4 ? (r == 7 ? 8 : 4) : r >= 2 ? (r == 3 ? 4 : 2) : 1;
            int kind = na == 1 ? 0 : na == 2 ? 1 : na == 4 ? 2 : na == 8 ? 3 : 4;
            vgs.push_back({kind, b0, first});
            first += na;
            r -= std::min(r, na);
        }
    }
    // passes: groups of one kind, in column order within the kind
    std::vector<int> order(vgs.size());
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return vgs[a].kind < vgs[b].kind; });
    std::vector<int> pairpos((size_t)M1 * P, -1);  // (m, nu) -> place in the per-warp area
    cs = ColSched{};
    std::vector<int> kinds;
    for (int k : order) {
        const VG& v = vgs[k];
        const int na = cols_na(v.kind);
        kinds.push_back(v.kind);
        cs.vgcol.push_back(v.col);
        cs.vgsrc.push_back((int)cs.src.size());
        for (int s = 0; s < na; ++s)
            for (int L = 0; L < 32; ++L) {
                const int c = v.col + L;
                const int t = v.first + s;
                int m = 31;
                if (c < P && t < (int)terms[c].size()) {
                    m = terms[c][t];
                    pairpos[(size_t)m * P + c] = (int)cs.vgcol.size() - 1 + (s << 20);
                }
                cs.src.push_back((unsigned char)m);
            }
    }
    for (int es : {4, 8}) {
        auto& pass = es == 4 ? cs.pass : cs.pass64;
        for (size_t k = 0; k < kinds.size();) {
            const int kind = kinds[k], gp = cols_gp(kind, es);
            int ng = 0;
            while (k + ng < kinds.size() && kinds[k + ng] == kind && ng < gp) ++ng;
            pass.push_back(make_int4(kind, (int)k, ng, 0));
            k += ng;
        }
    }
    // per precision: the pass and place of every pair, then the entries of each output
    // column (K_0 pair with g = 1, then the G entries, in the pair form's order) by pass
    for (int es : {4, 8}) {
        const auto& pass = es == 4 ? cs.pass : cs.pass64;
        std::vector<int> vpass(cs.vgcol.size()), vg_in(cs.vgcol.size());
        for (size_t p = 0; p < pass.size(); ++p)
            for (int g = 0; g < pass[p].z; ++g) {
                vpass[pass[p].y + g] = (int)p;
                vg_in[pass[p].y + g] = g;
            }
        std::vector<std::vector<std::pair<int, double>>> lists(pass.size() * 32);
        for (int mu = 0; mu < P; ++mu)
            for (int e = h.combptr[mu]; e < h.combptr[mu + 1]; ++e) {
                const int q = h.qtab[h.combq[e]], m = q >> 16, nu = q & 0xffff;
                const int pp = pairpos[(size_t)m * P + nu], vg = pp & 0xfffff, sl = pp >> 20;
                const int na = cols_na(pass[vpass[vg]].x);
                const int place = (vg_in[vg] * na + sl) * 32 + (nu & 31);
                lists[(size_t)vpass[vg] * 32 + (mu & 31)].push_back({((mu >> 5) << 16) | place, h.combg[e]});
            }
        auto& ept = es == 4 ? cs.ept32 : cs.ept64;
        auto& eidx = es == 4 ? cs.eidx32 : cs.eidx64;
        auto& eg = es == 4 ? cs.eg32 : cs.eg64;
        ept.assign(lists.size() + 1, 0);
        for (size_t l = 0; l < lists.size(); ++l) {
            for (const auto& en : lists[l]) {
                eidx.push_back(en.first);
                eg.push_back(en.second);
            }
            ept[l + 1] = (int)eidx.size();
        }
    }
}

// ---- on-disk tuning cache: the launch shapes chosen for a set of problem shapes on a
// device model, so that a later finalize of the same batch skips the timing sweep.
// One line per entry: "<key hash> wpb qt bps wpb32 qt32 pf32 pf64 wpb64c"; the file is
// SGFEM_TUNE_CACHE, else $XDG_CACHE_HOME/extendableasgfem_gb300/batch_tuning.txt, else
// $HOME/.cache/extendableasgfem_gb300/batch_tuning.txt ("off" disables it).
struct TuneEntry {
    int wpb, qt, bps, wpb32, qt32, pf32, pf64, wpb64c;
};

std::string tune_path() {
    const char* e = getenv("SGFEM_TUNE_CACHE");
    if (e) return std::string(e) == "off" ? std::string() : std::string(e);
    std::string dir;
    if (const char* x = getenv("XDG_CACHE_HOME")) dir = x;
    else if (const char* h = getenv("HOME")) dir = std::string(h) + "/.cache";
    else return std::string();
    mkdir(dir.c_str(), 0755);  // may exist already
    dir += "/extendableasgfem_gb300";
    mkdir(dir.c_str(), 0755);
    return dir + "/batch_tuning.txt";
}

std::string tune_key(const sgfem_batch* b) {
    cudaDeviceProp pr{};
    cudaGetDeviceProperties(&pr, b->device);
    std::string k = std::string(pr.name) + "|" + std::to_string(pr.multiProcessorCount) + "|v2";
    for (const auto& h : b->hp)
        k += "|" + std::to_string(h.n) + "," + std::to_string(h.P) + "," + std::to_string(h.M1) + "," +
             std::to_string(h.col.size()) + "," + std::to_string(h.qtab.size()) + "," + std::to_string(h.nl);
    uint64_t f = 1469598103934665603ull;  // FNV-1a
    for (unsigned char c : k) {
        f ^= c;
        f *= 1099511628211ull;
    }
    char buf[48];
    snprintf(buf, sizeof(buf), "%016llx-%zu", (unsigned long long)f, b->hp.size());
    return buf;
}

bool tune_lookup(const std::string& path, const std::string& key, TuneEntry& e) {
    if (path.empty()) return false;
    FILE* f = fopen(path.c_str(), "r");
    if (!f) return false;
    char k[64];
    TuneEntry t{};
    bool found = false;
    while (fscanf(f, "%63s %d %d %d %d %d %d %d %d", k, &t.wpb, &t.qt, &t.bps, &t.wpb32, &t.qt32, &t.pf32, &t.pf64,
                  &t.wpb64c) == 9)
        if (key == k) {
            e = t;
            found = true;  // the last entry for a key wins
        }
    fclose(f);
    return found;
}

void tune_store(const std::string& path, const std::string& key, const TuneEntry& e) {
    if (path.empty()) return;
    FILE* f = fopen(path.c_str(), "a");
    if (!f) return;
    fprintf(f, "%s %d %d %d %d %d %d %d %d\n", key.c_str(), e.wpb, e.qt, e.bps, e.wpb32, e.qt32, e.pf32, e.pf64,
            e.wpb64c);
    fclose(f);
}

}  // namespace

extern "C" int sgfem_batch_create(sgfem_batch** out, int device) {
    if (!out) return SGFEM_ERR_ARGUMENT;
    *out = nullptr;
    sgfem_batch* b = new sgfem_batch();
    b->device = device;
    if (cudaSetDevice(device) != cudaSuccess || cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreate(&b->ev0) != cudaSuccess || cudaEventCreate(&b->ev1) != cudaSuccess) {
        delete b;
        return SGFEM_ERR_CUDA;
    }
    cudaDeviceGetAttribute(&b->num_sms, cudaDevAttrMultiProcessorCount, device);
    *out = b;
    return SGFEM_OK;
}

extern "C" int sgfem_batch_destroy(sgfem_batch* b) {
    if (!b) return SGFEM_OK;
    cudaSetDevice(b->device);
    if (b->stream) cudaStreamSynchronize(b->stream);
    for (void* p : b->owned) cudaFree(p);
    if (b->ev0) cudaEventDestroy(b->ev0);
    if (b->ev1) cudaEventDestroy(b->ev1);
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
    return SGFEM_OK;
}

extern "C" const char* sgfem_batch_last_error(const sgfem_batch* b) { return b ? b->err.c_str() : "null batch"; }

extern "C" int sgfem_batch_add(sgfem_batch* b, int64_t n, int64_t M, int64_t P, const int64_t* colptr,
                               const int64_t* rowval, const double* vals, const int64_t* Gcolptr,
                               const int64_t* Growval, const double* Gval, int64_t nbd, const int64_t* bdofs,
                               const double* b0) {
    if (!b) return SGFEM_ERR_ARGUMENT;
    if (b->finalized) return bfail(b, SGFEM_ERR_STATE, "batch already finalized");
    if (n <= 0 || n > (1 << 30) || M < 0 || M > 255 || P <= 0 || P > 32767 || !colptr || !rowval || !vals ||
        !Gcolptr || (nbd > 0 && !bdofs) || !b0)
        return bfail(b, SGFEM_ERR_ARGUMENT, "sgfem_batch_add: bad arguments (M <= 255, P <= 32767)");
    sgfem_batch::HostProb h;
    h.n = (int)n;
    h.P = (int)P;
    h.M1 = (int)M + 1;
    h.ld = (int)((P + 3) / 4 * 4);
    const int64_t nnz = colptr[n] - 1;
    if (colptr[0] != 1 || nnz < 0) return bfail(b, SGFEM_ERR_ARGUMENT, "colptr must be 1-based");
    // CSC (shared pattern) -> CSR; vals is (M+1) x nnz column-major: value of block m at [m * nnz + k]
    std::vector<int> cnt(n + 1, 0);
    for (int64_t k = 0; k < nnz; ++k) {
        const int64_t r = rowval[k] - 1;
        if (r < 0 || r >= n) return bfail(b, SGFEM_ERR_ARGUMENT, "rowval out of range");
        cnt[r + 1]++;
    }
    for (int64_t i = 0; i < n; ++i) cnt[i + 1] += cnt[i];
    h.rowptr = cnt;
    h.col.assign(nnz, 0);
    h.vals.assign((size_t)nnz * h.M1, 0.0);
    std::vector<int> fill(cnt.begin(), cnt.end() - 1);
    for (int64_t j = 0; j < n; ++j)
        for (int64_t k = colptr[j] - 1; k < colptr[j + 1] - 1; ++k) {
            const int r = (int)(rowval[k] - 1);
            const int at = fill[r]++;
            h.col[at] = (int)j;
            for (int m = 0; m < h.M1; ++m) h.vals[(size_t)at * h.M1 + m] = vals[(size_t)m * nnz + k];
        }
    h.bmask.assign(n, 0);
    for (int64_t t = 0; t < nbd; ++t) {
        const int64_t d = bdofs[t] - 1;
        if (d < 0 || d >= n) return bfail(b, SGFEM_ERR_ARGUMENT, "boundary dof out of range");
        h.bmask[d] = 1;
    }
    h.dinv.assign(n, 0.0);
    for (int i = 0; i < n; ++i) {
        if (h.bmask[i]) continue;
        double dg = 0.0;
        for (int k = h.rowptr[i]; k < h.rowptr[i + 1]; ++k)
            if (h.col[k] == i) dg += h.vals[(size_t)k * h.M1];
        if (!(dg > 0.0)) return bfail(b, SGFEM_ERR_ARGUMENT, "K_0 has a non-positive interior diagonal entry");
        h.dinv[i] = 1.0 / dg;
    }
    // coupling: pairs (0, nu) for all nu, then (m, nu) for nonzero columns of G_m; combination lists per mu
    if (Gcolptr[0] != 1) return bfail(b, SGFEM_ERR_ARGUMENT, "G colptr must be 1-based");
    std::vector<std::vector<char>> nzc(h.M1, std::vector<char>(P, 0));
    struct GE { int m, mu, nu; double g; };
    std::vector<GE> ges;
    for (int64_t nu = 0; nu < P; ++nu)
        for (int64_t k = Gcolptr[nu] - 1; k < Gcolptr[nu + 1] - 1; ++k) {
            const int64_t r = Growval[k] - 1;
            if (r < 0 || r >= M * P) return bfail(b, SGFEM_ERR_ARGUMENT, "G rowval out of range");
            if (Gval[k] == 0.0) continue;
            const int m = (int)(r / P) + 1, mu = (int)(r % P);
            nzc[m][nu] = 1;
            ges.push_back({m, mu, (int)nu, Gval[k]});
        }
    // pairs ordered by column nu, then term m: a pass of the apply over consecutive
    // pairs reads a narrow column range of each X row
    std::vector<int> qidx((size_t)h.M1 * P, -1);
    for (int nu = 0; nu < P; ++nu)
        for (int m = 0; m < h.M1; ++m)
            if (m == 0 || nzc[m][nu]) {
                qidx[(size_t)m * P + nu] = (int)h.qtab.size();
                h.qtab.push_back((m << 16) | nu);
            }
    // per output mode mu: its K_0 pair with g = 1 first, then the G entries in their order
    h.combptr.assign(P + 1, 0);
    std::stable_sort(ges.begin(), ges.end(), [](const GE& x, const GE& y) { return x.mu < y.mu; });
    size_t e0 = 0;
    for (int mu = 0; mu < P; ++mu) {
        h.combptr[mu + 1]++;
        h.combq.push_back(qidx[mu]);
        h.combg.push_back(1.0);
        for (; e0 < ges.size() && ges[e0].mu == mu; ++e0) {
            h.combptr[mu + 1]++;
            h.combq.push_back(qidx[(size_t)ges[e0].m * P + ges[e0].nu]);
            h.combg.push_back(ges[e0].g);
        }
    }
    for (int mu = 0; mu < P; ++mu) h.combptr[mu + 1] += h.combptr[mu];
    h.b0.assign(b0, b0 + n);
    h.work = (double)nnz * (double)h.qtab.size() + 4.0 * (double)n * h.ld;
    b->hp.push_back(std::move(h));
    return SGFEM_OK;
}

extern "C" int sgfem_batch_count(const sgfem_batch* b) { return b ? (int)b->hp.size() : 0; }

extern "C" int sgfem_batch_set_lattice(sgfem_batch* b, int i, int64_t nl) {
    if (!b) return SGFEM_ERR_ARGUMENT;
    if (b->finalized) return bfail(b, SGFEM_ERR_STATE, "batch already finalized");
    if (i < 0 || i >= (int)b->hp.size()) return bfail(b, SGFEM_ERR_ARGUMENT, "no such problem");
    auto& h = b->hp[i];
    if (nl < 2 || nl > 128 || (int64_t)h.n != (nl + 1) * (nl + 1))
        return bfail(b, SGFEM_ERR_ARGUMENT, "lattice: n must be (nl + 1)^2 with 2 <= nl <= 128");
    // interior rows are the lattice interior; a0 = mean interior diagonal / 4
    double dsum = 0.0;
    long long cnt = 0;
    for (int64_t r = 0; r < h.n; ++r) {
        const int64_t ix = r % (nl + 1), iy = r / (nl + 1);
        const bool interior = ix > 0 && ix < nl && iy > 0 && iy < nl;
        if (interior != !h.bmask[r]) return bfail(b, SGFEM_ERR_ARGUMENT, "lattice: Dirichlet rows are not the lattice boundary");
        if (interior) {
            dsum += 1.0 / h.dinv[r];
            ++cnt;
        }
    }
    h.a0 = cnt ? dsum / (4.0 * cnt) : 1.0;
    h.nl = (int)nl;
    return SGFEM_OK;
}

extern "C" int sgfem_batch_finalize(sgfem_batch* b) {
    if (!b) return SGFEM_ERR_ARGUMENT;
    if (b->finalized) return bfail(b, SGFEM_ERR_STATE, "batch already finalized");
    if (b->hp.empty()) return bfail(b, SGFEM_ERR_STATE, "no problems added");
    BCUDA(b, cudaSetDevice(b->device));
    const int B = (int)b->hp.size();
    std::vector<BProb> probs(B);
    long long voff = 0;
    for (int i = 0; i < B; ++i) {
        auto& h = b->hp[i];
        BProb& d = probs[i];
        d.n = h.n;
        d.P = h.P;
        d.ld = h.ld;
        d.M1 = h.M1;
        d.Qn = (int)h.qtab.size();
        d.voff = voff;
        voff += (long long)h.n * h.ld;
        SG_TRY(bupload(b, h.rowptr, (int**)&d.rowptr));
        SG_TRY(bupload(b, h.col, (int**)&d.col));
        SG_TRY(bupload(b, h.vals, (double**)&d.vals));
        SG_TRY(bupload(b, h.bmask, (unsigned char**)&d.bmask));
        SG_TRY(bupload(b, h.dinv, (double**)&d.dinv));
        SG_TRY(bupload(b, h.qtab, (int**)&d.qtab));
        SG_TRY(bupload(b, h.combptr, (int**)&d.combptr));
        SG_TRY(bupload(b, h.combq, (int**)&d.combq));
        SG_TRY(bupload(b, h.combg, (double**)&d.combg));
        {
            const std::vector<float> v32(h.vals.begin(), h.vals.end()), g32(h.combg.begin(), h.combg.end()),
                d32(h.dinv.begin(), h.dinv.end());
            SG_TRY(bupload(b, v32, (float**)&d.vals32));
            SG_TRY(bupload(b, g32, (float**)&d.combg32));
            SG_TRY(bupload(b, d32, (float**)&d.dinv32));
        }
        b->ldmax = std::max(b->ldmax, h.ld);
        b->m1max = std::max(b->m1max, h.M1);
        b->qnmax = std::max(b->qnmax, d.Qn);
    }
    // column-slot schedules (every problem needs M + 1 <= 31: lane 31 holds the zero value)
    b->cols_ok = b->m1max <= 31;
    if (const char* ea = getenv("SGFEM_BATCH_APPLY"))
        if (std::string(ea) == "pairs") b->cols_ok = false;
    for (int i = 0; i < B && b->cols_ok; ++i) {
        ColSched cs;
        build_cols(b->hp[i], cs);
        BProb& d = probs[i];
        d.npass = (int)cs.pass.size();
        d.npass64 = (int)cs.pass64.size();
        SG_TRY(bupload(b, cs.pass, (int4**)&d.cpass));
        SG_TRY(bupload(b, cs.pass64, (int4**)&d.cpass64));
        SG_TRY(bupload(b, cs.vgcol, (int**)&d.vgcol));
        SG_TRY(bupload(b, cs.vgsrc, (int**)&d.vgsrc));
        SG_TRY(bupload(b, cs.src, (unsigned char**)&d.src));
        SG_TRY(bupload(b, cs.ept32, (int**)&d.ept32));
        SG_TRY(bupload(b, cs.eidx32, (int**)&d.eidx32));
        SG_TRY(bupload(b, std::vector<float>(cs.eg32.begin(), cs.eg32.end()), (float**)&d.eg32));
        SG_TRY(bupload(b, cs.ept64, (int**)&d.ept64));
        SG_TRY(bupload(b, cs.eidx64, (int**)&d.eidx64));
        SG_TRY(bupload(b, cs.eg64, (double**)&d.eg64));
    }
    b->total = voff;
    const size_t vb = (size_t)voff * sizeof(double);
    SG_TRY(balloc(b, vb, (void**)&b->d_x));
    SG_TRY(balloc(b, vb, (void**)&b->d_b));
    SG_TRY(balloc(b, vb, (void**)&b->d_r));
    SG_TRY(balloc(b, vb, (void**)&b->d_p));
    SG_TRY(balloc(b, vb, (void**)&b->d_q));
    SG_TRY(balloc(b, (size_t)B * sizeof(KrylovScalars), (void**)&b->d_scal));
    SG_TRY(balloc(b, vb, (void**)&b->d_z));
    BCUDA(b, cudaMemset(b->d_z, 0, vb));
    const size_t vb32 = (size_t)voff * sizeof(float);
    SG_TRY(balloc(b, vb32, (void**)&b->d_r32));
    SG_TRY(balloc(b, vb32, (void**)&b->d_p32));
    SG_TRY(balloc(b, vb32, (void**)&b->d_q32));
    SG_TRY(balloc(b, vb32, (void**)&b->d_z32));
    SG_TRY(balloc(b, vb, (void**)&b->d_d64));
    SG_TRY(balloc(b, (size_t)B * sizeof(double), (void**)&b->d_want));
    {
        // sine-transform preconditioner: per-problem (nl, a0), the split sine tables of each
        // lattice size (k_bdst; offsets multiples of 16 floats) and one block per
        // (problem, interior line)
        std::vector<int2> lat(B, make_int2(0, 0));
        std::vector<int2> map;
        std::vector<int> soff(B, 0), toff(129, -1);
        std::vector<float> stab;
        size_t smax = 0;
        for (int i = 0; i < B; ++i) {
            const auto& h = b->hp[i];
            if (h.nl <= 0) continue;
            float a0f = (float)h.a0;
            int bits;
            std::memcpy(&bits, &a0f, sizeof(int));
            lat[i] = make_int2(h.nl, bits);
            const DstShape q = dst_shape(h.nl);
            if (toff[h.nl] < 0) {
                toff[h.nl] = (int)stab.size();
                dst_tables(h.nl, stab);
            }
            soff[i] = toff[h.nl];
            for (int line = 1; line <= q.N; ++line) map.push_back(make_int2(i, line));
            smax = std::max(smax, ((size_t)q.tab + (size_t)q.N * q.cw) * sizeof(float));
        }
        SG_TRY(bupload(b, lat, &b->d_lat));
        b->ndst = (int)map.size();
        if (b->ndst > 0) {
            SG_TRY(bupload(b, map, &b->d_dstmap));
            SG_TRY(bupload(b, soff, &b->d_soff));
            SG_TRY(bupload(b, stab, &b->d_stab));
            SG_TRY(balloc(b, (size_t)voff * sizeof(float), (void**)&b->d_t));
            b->dst_smem = smax;
            if (smax > 48 * 1024) {
                BCUDA(b, cudaFuncSetAttribute(k_bdst<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smax));
                BCUDA(b, cudaFuncSetAttribute(k_bdst<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smax));
            }
        }
    }
    BCUDA(b, cudaMemset(b->d_x, 0, vb));
    BCUDA(b, cudaMemset(b->d_p, 0, vb));
    b->h_scal.assign(B, KrylovScalars{});
    BCUDA(b, cudaMemset(b->d_scal, 0, (size_t)B * sizeof(KrylovScalars)));

    // ---- autotune the apply: warps per block x pairs per lane x blocks per SM
    struct Cand { int wpb, qt, bps; };
    std::vector<Cand> cands;
    // 2 warps/block, 4 pairs per lane and 4 blocks per SM lost on every batch measured
    for (int wpb : {4, 8})
        for (int qt : {8, 16})
            for (int bps : {8, 16}) cands.push_back({wpb, qt, bps});
    int dev_smem = 0;
    cudaDeviceGetAttribute(&dev_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, b->device);
    float best = 1e30f;
    Cand bestc{0, 0, 0};
    std::vector<int> bprob;
    BProb* d_probs = nullptr;
    SG_TRY(balloc(b, (size_t)B * sizeof(BProb), (void**)&d_probs));
    b->d_probs = d_probs;
    int* d_bmap = nullptr;
    const int max_blocks = b->num_sms * 16 + B;
    SG_TRY(balloc(b, (size_t)std::max(max_blocks, 1) * 4 * sizeof(int), (void**)&d_bmap));
    b->d_bprob = d_bmap;
    SG_TRY(balloc(b, (size_t)std::max(max_blocks, 1) * 4 * sizeof(int), (void**)&b->d_vorder));
    SG_TRY(balloc(b, sizeof(int), (void**)&b->d_wq));
    SG_TRY(balloc(b, (size_t)std::max(max_blocks, 1) * 4 * sizeof(double), (void**)&b->d_part));
    std::string log;
    // tuning cache: a batch of the same shapes on the same device model was tuned before
    const std::string tpath = tune_path(), tkey = tune_key(b);
    TuneEntry te{};
    bool hit = tune_lookup(tpath, tkey, te);
    if (hit) {
        const bool ok64 = (te.wpb == 4 || te.wpb == 8) && (te.qt == 8 || te.qt == 16) && te.bps >= 1 &&
                          te.bps <= 16 && (int)apply_smem(b, te.wpb) <= dev_smem;
        const bool ok32 = (te.wpb32 == 4 || te.wpb32 == 8) && (te.qt32 == 16 || te.qt32 == 32) &&
                          te.pf32 >= 0 && te.pf32 <= 6 && te.pf32 != 5 &&
                          (!(te.pf32 & 4) || b->cols_ok) &&
                          (!(te.pf32 & 1) || (b->ldmax <= 32 * BPC && b->m1max <= 32 * BPV)) &&
                          (int)apply_smem<float>(b, te.wpb32, te.pf32) <= dev_smem;
        const bool okc64 = te.pf64 == 0 || (te.pf64 == 4 && b->cols_ok && (te.wpb64c == 4 || te.wpb64c == 8) &&
                                            (int)apply_smem<double>(b, te.wpb64c, 4) <= dev_smem);
        hit = ok64 && ok32 && okc64;
    }
    if (hit) {
        BCUDA(b, set_apply_smem<double>(0, te.qt, apply_smem(b, te.wpb)));
        BCUDA(b, set_apply_smem<float>(te.pf32, te.qt32, apply_smem<float>(b, te.wpb32, te.pf32)));
        if (te.pf64 & 4) BCUDA(b, set_apply_smem<double>(4, 0, apply_smem<double>(b, te.wpb64c, 4)));
        best = 0.f;
        bestc = Cand{te.wpb, te.qt, te.bps};
        b->wpb32 = te.wpb32;
        b->qt32 = te.qt32;
        b->pf32 = te.pf32;
        b->pf64 = te.pf64;
        b->wpb64c = te.wpb64c;
        log = "from the tuning cache " + tpath + "; ";
    }
    for (const Cand& c : cands) {
        if (hit) break;
        const size_t smem = apply_smem(b, c.wpb);
        if ((int)smem > dev_smem) continue;
        if (smem > 48 * 1024) {
            cudaError_t e = c.qt == 8 ? cudaFuncSetAttribute(k_bapply<double, 8>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)
                                      : cudaFuncSetAttribute(k_bapply<double, 16>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            if (e != cudaSuccess) {
                cudaGetLastError();
                continue;
            }
        }
        SG_TRY(build_map(b, b->num_sms * c.bps, probs, bprob));
        if ((int)bprob.size() > max_blocks * 4) continue;
        SG_TRY(upload_map(b, probs, bprob));
        SG_TRY(launch_apply<double>(b, c.wpb, c.qt, b->d_p, b->d_q, b->d_part, nullptr));  // warm-up
        BCUDA(b, cudaEventRecord(b->ev0, b->stream));
        SG_TRY(launch_apply<double>(b, c.wpb, c.qt, b->d_p, b->d_q, b->d_part, nullptr));
        BCUDA(b, cudaEventRecord(b->ev1, b->stream));
        BCUDA(b, cudaEventSynchronize(b->ev1));
        float ms = 0.f;
        BCUDA(b, cudaEventElapsedTime(&ms, b->ev0, b->ev1));
        char buf[96];
        snprintf(buf, sizeof(buf), "%dw/%dq/%dbps:%.3fms ", c.wpb, c.qt, c.bps, ms);
        log += buf;
        if (ms < best) {
            best = ms;
            bestc = c;
        }
    }
    if (bestc.wpb == 0) return bfail(b, SGFEM_ERR_UNSUPPORTED, "no apply launch shape fits the shared memory");
    b->wpb = bestc.wpb;
    b->qt = bestc.qt;
    SG_TRY(build_map(b, b->num_sms * bestc.bps, probs, bprob));
    SG_TRY(upload_map(b, probs, bprob));
    // FP64 apply in the column-slot form on the same block map (residuals of the mixed
    // solve, every iteration of the FP64 solve)
    std::string log64c;
    for (int wpb : {4, 8}) {
        if (hit || !b->cols_ok) break;
        const size_t smem = apply_smem<double>(b, wpb, 4);
        if ((int)smem > dev_smem) continue;
        if (set_apply_smem<double>(4, 0, smem) != cudaSuccess) {
            cudaGetLastError();
            continue;
        }
        SG_TRY(launch_apply<double>(b, wpb, 0, b->d_p, b->d_q, b->d_part, nullptr, 4));
        BCUDA(b, cudaEventRecord(b->ev0, b->stream));
        SG_TRY(launch_apply<double>(b, wpb, 0, b->d_p, b->d_q, b->d_part, nullptr, 4));
        BCUDA(b, cudaEventRecord(b->ev1, b->stream));
        BCUDA(b, cudaEventSynchronize(b->ev1));
        float ms = 0.f;
        BCUDA(b, cudaEventElapsedTime(&ms, b->ev0, b->ev1));
        char buf64[64];
        snprintf(buf64, sizeof(buf64), "cols %dw:%.3fms ", wpb, ms);
        log64c += buf64;
        if (ms < best) {
            best = ms;
            b->pf64 = 4;
            b->wpb64c = wpb;
        }
    }
    // FP32 apply of the mixed solve on the same block map: more pairs per pass amortise
    // the staging of each X row (LSU-bound rather than FP64-bound); the column-slot form
    // (pf 4, 6) reads each X row once per column group and nonzero
    std::string log32;
    float best32 = 1e30f;
    for (int pf : {0, 1, 2, 3, 4, 6})
        for (int wpb : {4, 8})
            for (int qt : {16, 32}) {
                if (hit) break;
                if ((pf & 1) && (b->ldmax > 32 * BPC || b->m1max > 32 * BPV)) continue;
                if ((pf & 4) && (!b->cols_ok || qt != 16)) continue;
                const size_t smem = apply_smem<float>(b, wpb, pf);
                if ((int)smem > dev_smem) continue;
                {  // the register budget of the variant must allow the block size
                    cudaFuncAttributes fa{};
                    const cudaError_t ea = cudaFuncGetAttributes(&fa, apply_kernel<float>(pf, qt));
                    if (ea != cudaSuccess || fa.maxThreadsPerBlock < wpb * 32) {
                        cudaGetLastError();
                        continue;
                    }
                }
                if (set_apply_smem<float>(pf, qt, smem) != cudaSuccess) {
                    cudaGetLastError();
                    continue;
                }
                SG_TRY(launch_apply<float>(b, wpb, qt, b->d_p32, b->d_q32, b->d_part, nullptr, pf));
                BCUDA(b, cudaEventRecord(b->ev0, b->stream));
                for (int r = 0; r < 2; ++r)
                    SG_TRY(launch_apply<float>(b, wpb, qt, b->d_p32, b->d_q32, b->d_part, nullptr, pf));
                BCUDA(b, cudaEventRecord(b->ev1, b->stream));
                BCUDA(b, cudaEventSynchronize(b->ev1));
                float ms = 0.f;
                BCUDA(b, cudaEventElapsedTime(&ms, b->ev0, b->ev1));
                char buf32[96];
                if (pf & 4)
                    snprintf(buf32, sizeof(buf32), "%scols %dw:%.3fms ", (pf & 2) ? "queue " : "", wpb, ms / 2);
                else
                    snprintf(buf32, sizeof(buf32), "%s%s%dw/%dq:%.3fms ", (pf & 2) ? "queue " : "",
                             (pf & 1) ? "prefetch " : "", wpb, qt, ms / 2);
                log32 += buf32;
                if (ms < best32) {
                    best32 = ms;
                    b->wpb32 = wpb;
                    b->qt32 = qt;
                    b->pf32 = pf;
                }
            }
    if (!hit)
        tune_store(tpath, tkey, TuneEntry{b->wpb, b->qt, bestc.bps, b->wpb32, b->qt32, b->pf32, b->pf64, b->wpb64c});
    // SGFEM_BATCH_APPLY=cols: the column-slot form for both precisions (pairs: never, at finalize)
    if (const char* ea = getenv("SGFEM_BATCH_APPLY"))
        if (std::string(ea) == "cols" && b->cols_ok) {
            if (!(b->pf32 & 4)) {
                b->pf32 = 4;
                b->qt32 = 16;
                b->wpb32 = (int)apply_smem<float>(b, 8, 4) <= dev_smem ? 8 : 4;
            }
            if (!(b->pf64 & 4)) {
                b->pf64 = 4;
                b->wpb64c = (int)apply_smem<double>(b, 8, 4) <= dev_smem ? 8 : 4;
            }
            BCUDA(b, set_apply_smem<float>(4, 16, apply_smem<float>(b, b->wpb32, 4)));
            BCUDA(b, set_apply_smem<double>(4, 0, apply_smem<double>(b, b->wpb64c, 4)));
        }
    if (const char* q = getenv("SGFEM_BATCH_QUEUE"))  // 1 / 0: the FP32 apply over the work queue or not
        b->pf32 = atoi(q) ? (b->pf32 | 2) : (b->pf32 & ~2);
    if (b->pf32 & 1) {
        // the prefetching pair form needs its shared-memory opt-in like the others
        BCUDA(b, set_apply_smem<float>(b->pf32, b->qt32, apply_smem<float>(b, b->wpb32, b->pf32)));
    }
    char buf[320];
    const char* f32form = (b->pf32 & 4) ? ((b->pf32 & 2) ? "work queue, column slots, " : "column slots, ")
                          : b->pf32 == 3 ? "work queue, prefetch, " : b->pf32 == 2 ? "work queue, " : b->pf32 ? "prefetch, " : "";
    if (b->pf64 & 4)
        snprintf(buf, sizeof(buf), "chosen column slots, %d warps/block, %d blocks (FP32: %s%d warps/block, %d pairs/lane); ",
                 b->wpb64c, b->blocks, f32form, b->wpb32, b->qt32 * 32);
    else
        snprintf(buf, sizeof(buf), "chosen %d warps/block, %d pairs/lane, %d blocks (FP32: %s%d warps/block, %d pairs/lane); ",
                 b->wpb, b->qt * 32, b->blocks, f32form, b->wpb32, b->qt32 * 32);
    log += log64c;
    b->tuning = buf + log + "FP32 " + log32;
    b->finalized = true;
    return SGFEM_OK;
}

extern "C" const char* sgfem_batch_tuning(const sgfem_batch* b) { return b ? b->tuning.c_str() : ""; }

// Host check of the column-slot schedule: the problem is added as sgfem_batch_add does
// (no device work), its schedule built as at finalize, and the sums of k_bapply_cols
// evaluated on the host in FP64 with the FP32 (precision 1) or FP64 (precision 0) pass
// structure: every pass's pair sums (slot sources, clamped columns, padding groups) go
// to the pass area and each output column takes its pass's entries.  X and Y are n x P
// column-major (the SGFEVector layout); Dirichlet rows of Y are zero.
extern "C" int sgfem_batch_host_apply(int64_t n, int64_t M, int64_t P, const int64_t* colptr, const int64_t* rowval,
                                      const double* vals, const int64_t* Gcolptr, const int64_t* Growval,
                                      const double* Gval, int64_t nbd, const int64_t* bdofs, int precision,
                                      const double* X, double* Y, char* msg, int msglen) {
    auto say = [&](const std::string& t) {
        if (msg && msglen > 0) snprintf(msg, (size_t)msglen, "%s", t.c_str());
    };
    if (!X || !Y || (precision != 0 && precision != 1)) return SGFEM_ERR_ARGUMENT;
    std::vector<double> b0(n > 0 ? (size_t)n : 1, 0.0);
    sgfem_batch tmp;
    const int rc = sgfem_batch_add(&tmp, n, M, P, colptr, rowval, vals, Gcolptr, Growval, Gval, nbd, bdofs, b0.data());
    if (rc != SGFEM_OK) {
        say(tmp.err);
        return rc;
    }
    const auto& h = tmp.hp[0];
    if (h.M1 > 31) {
        say("the column-slot form needs M + 1 <= 31");
        return SGFEM_ERR_UNSUPPORTED;
    }
    ColSched cs;
    build_cols(h, cs);
    const int es = precision == 1 ? 4 : 8;
    const auto& pass = es == 4 ? cs.pass : cs.pass64;
    const auto& ept = es == 4 ? cs.ept32 : cs.ept64;
    const auto& eidx = es == 4 ? cs.eidx32 : cs.eidx64;
    const auto& eg = es == 4 ? cs.eg32 : cs.eg64;
    const int ld = h.ld, M1 = h.M1;
    std::vector<double> area(512), ys(ld);
    long long slots = 0;
    for (const auto& p : pass) {
        if (p.z < 1 || p.z > cols_gp(p.x, es) || cols_na(p.x) * p.z * 32 > 512) {
            say("pass shape outside the kernel's limits");
            return SGFEM_ERR_UNSUPPORTED;
        }
        slots += (long long)cols_na(p.x) * p.z * 32;
    }
    for (int64_t i = 0; i < n; ++i) {
        std::fill(ys.begin(), ys.end(), 0.0);
        if (!h.bmask[i]) {
            for (size_t pp = 0; pp < pass.size(); ++pp) {
                const int4 p = pass[pp];
                const int na = cols_na(p.x);
                std::fill(area.begin(), area.end(), 0.0);
                for (int g = 0; g < p.z; ++g) {
                    const int vg = p.y + g;
                    for (int L = 0; L < 32; ++L) {
                        const int c = std::min(cs.vgcol[vg] + L, ld - 1);
                        for (int sl = 0; sl < na; ++sl) {
                            const int m = cs.src[(size_t)cs.vgsrc[vg] + 32 * sl + L];
                            double f = 0.0;
                            for (int k = h.rowptr[i]; k < h.rowptr[i + 1]; ++k) {
                                const int j = h.col[k];
                                const double xv = c < P ? X[(size_t)c * n + j] : 0.0;
                                f += (m < M1 ? h.vals[(size_t)k * M1 + m] : 0.0) * xv;
                            }
                            area[(size_t)(g * na + sl) * 32 + L] = f;
                        }
                    }
                }
                for (int L = 0; L < 32; ++L)
                    for (int e = ept[pp * 32 + L]; e < ept[pp * 32 + L + 1]; ++e) {
                        const int v = eidx[e];
                        ys[(size_t)(v >> 16) * 32 + L] += eg[e] * area[v & 0xffff];
                    }
            }
        }
        for (int64_t mu = 0; mu < P; ++mu) Y[(size_t)mu * n + i] = ys[mu];
    }
    char buf[160];
    snprintf(buf, sizeof(buf), "%zu passes, %zu groups, %.3f slots per pair (%lld slots, %zu pairs)", pass.size(),
             cs.vgcol.size(), (double)slots / (double)h.qtab.size(), slots, h.qtab.size());
    say(buf);
    return SGFEM_OK;
}

// Host check of the batch sine transform: y = S x (S_ik = sin(pi i k / nl), i, k = 1..nl-1)
// for ncols lines x (N x ncols, column-major), computed as k_bdst computes it from the
// split tables (the pair (x_k, x_{nl-k}) turned into (u_k, v_k), odd outputs from u and
// the middle point, even outputs from v), in FP64 with the FP32 table values.
extern "C" int sgfem_batch_host_dst(int64_t nl, int64_t ncols, const double* x, double* y) {
    if (nl < 2 || nl > 128 || ncols < 0 || (ncols > 0 && (!x || !y))) return SGFEM_ERR_ARGUMENT;
    const DstShape q = dst_shape((int)nl);
    std::vector<float> tab;
    dst_tables((int)nl, tab);
    if ((int)tab.size() != q.tab) return SGFEM_ERR_UNSUPPORTED;
    const float* TO = tab.data();
    const float* TE = TO + (size_t)q.HU * q.NOP;
    std::vector<double> t(q.N);
    for (int64_t c = 0; c < ncols; ++c) {
        const double* xc = x + (size_t)c * q.N;
        double* yc = y + (size_t)c * q.N;
        for (int k = 0; k < q.N; ++k) t[k] = xc[k];
        for (int k = 1; k <= q.H; ++k) {
            const double a = t[k - 1], b = t[nl - k - 1];
            t[k - 1] = a + b;
            t[nl - k - 1] = a - b;
        }
        for (int j = 0; j < q.no; ++j) {
            double s = 0.0;
            for (int r = 0; r < q.HU; ++r) s += (double)TO[(size_t)r * q.NOP + j] * t[r];
            yc[2 * j] = s;
        }
        for (int j = 0; j < q.ne; ++j) {
            double s = 0.0;
            for (int r = 0; r < q.H; ++r) s += (double)TE[(size_t)r * q.NEP + j] * t[q.HU + r];
            yc[2 * j + 1] = s;
        }
    }
    return SGFEM_OK;
}

namespace {

// z = B r (sine transform on lattice problems, Jacobi on the others), rho = r'z, beta, p = z + beta p
// the PCG vectors of one precision: FP64 (x, r, p, q, z) or the FP32 inner set with the FP64 accumulator
template <typename T, typename TX>
struct BVecs {
    TX* x;
    T *r, *p, *q, *z;
};

template <typename T, typename TX>
int batch_precondition(sgfem_batch* b, const BVecs<T, TX>& v, int maxit) {
    const int B = (int)b->hp.size();
    k_bjz<T><<<b->blocks, BT, 0, b->stream>>>(b->d_probs, b->d_bprob, b->d_lat, v.r, v.z, b->d_scal);
    BLAUNCHED(b);
    if (b->ndst > 0)
        for (int pass = 0; pass < 3; ++pass) {
            k_bdst<T><<<b->ndst, DST_WARPS * 32, b->dst_smem, b->stream>>>(b->d_probs, b->d_dstmap, b->d_lat, b->d_soff,
                                                                             b->d_stab, pass, v.r, b->d_t,
                                                               v.z, b->d_scal);
            BLAUNCHED(b);
        }
    k_brz<T><<<b->blocks, BT, 0, b->stream>>>(b->d_probs, b->d_bprob, v.r, v.z, b->d_scal, b->d_part);
    BLAUNCHED(b);
    k_bfin<<<B, BT, 0, b->stream>>>(b->d_probs, b->d_part, b->d_scal, BF_BETA, 0.0, maxit);
    BLAUNCHED(b);
    k_bpz<T><<<b->blocks, BT, 0, b->stream>>>(b->d_probs, b->d_bprob, v.z, v.p, b->d_scal);
    BLAUNCHED(b);
    return SGFEM_OK;
}

template <typename T, typename TX>
int batch_iteration(sgfem_batch* b, const BVecs<T, TX>& v, int maxit) {
    const int B = (int)b->hp.size();
    if constexpr (sizeof(T) == 4)
        SG_TRY(launch_apply<T>(b, b->wpb32, b->qt32, v.p, v.q, b->d_part, b->d_scal, b->pf32));
    else
        SG_TRY(apply64(b, v.p, v.q, b->d_part, b->d_scal));
    k_bfin<<<B, BT, 0, b->stream>>>(b->d_probs, b->d_part, b->d_scal, BF_ALPHA, 0.0, maxit);
    BLAUNCHED(b);
    k_bupdate<T, TX><<<b->blocks, BT, 0, b->stream>>>(b->d_probs, b->d_bprob, v.x, v.p, v.r, v.q, b->d_scal,
                                                      b->d_part);
    BLAUNCHED(b);
    k_bfin<<<B, BT, 0, b->stream>>>(b->d_probs, b->d_part, b->d_scal, BF_RR, 0.0, maxit);
    BLAUNCHED(b);
    return batch_precondition<T, TX>(b, v, maxit);
}

// PCG on all problems from the residual in v.r (x = 0 in v.x for the problems that run):
// scalars reset (done kept for problems marked done in h_scal), tolerances from
// BF_TOL over the Jacobi partials of ||r||^2 (want per problem, or rtol2), then
// check_every iterations per graph replay until every problem is done.
template <typename T, typename TX>
int batch_pcg(sgfem_batch* b, const BVecs<T, TX>& v, const double* want, double rtol2, int maxit, int check_every,
              int* replays) {
    const int B = (int)b->hp.size();
    BCUDA(b, cudaMemcpyAsync(b->d_scal, b->h_scal.data(), (size_t)B * sizeof(KrylovScalars), cudaMemcpyHostToDevice,
                             b->stream));
    k_bjacobi<T><<<b->blocks, BT, 0, b->stream>>>(b->d_probs, b->d_bprob, v.r, v.p, b->d_scal, b->d_part, 2);
    BLAUNCHED(b);
    k_bfin<<<B, BT, 0, b->stream>>>(b->d_probs, b->d_part, b->d_scal, BF_TOL, rtol2, maxit, want);
    BLAUNCHED(b);
    BCUDA(b, cudaMemsetAsync(v.p, 0, (size_t)b->total * sizeof(T), b->stream));
    BCUDA(b, cudaMemsetAsync(v.z, 0, (size_t)b->total * sizeof(T), b->stream));
    SG_TRY((batch_precondition<T, TX>(b, v, maxit)));
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    BCUDA(b, cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
    const long long before = b->launches;
    int st = SGFEM_OK;
    for (int k = 0; k < check_every && st == SGFEM_OK; ++k) st = batch_iteration<T, TX>(b, v, maxit);
    const long long per_graph = b->launches - before;
    b->launches = before;
    cudaError_t ce = cudaStreamEndCapture(b->stream, &graph);
    if (st != SGFEM_OK || ce != cudaSuccess) {
        if (graph) cudaGraphDestroy(graph);
        return st != SGFEM_OK ? st : bfail(b, SGFEM_ERR_CUDA, "graph capture failed");
    }
    ce = cudaGraphInstantiate(&exec, graph, 0);
    while (ce == cudaSuccess) {
        ce = cudaMemcpyAsync(b->h_scal.data(), b->d_scal, (size_t)B * sizeof(KrylovScalars), cudaMemcpyDeviceToHost,
                             b->stream);
        if (ce == cudaSuccess) ce = cudaStreamSynchronize(b->stream);
        if (ce != cudaSuccess) break;
        bool all = true;
        for (auto& s : b->h_scal) all = all && s.done;
        if (all) break;
        ce = cudaGraphLaunch(exec, b->stream);
        b->launches += per_graph;
        ++*replays;
    }
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    if (ce != cudaSuccess) return bfail(b, SGFEM_ERR_CUDA, std::string("batch iteration: ") + cudaGetErrorString(ce));
    return SGFEM_OK;
}

}  // namespace

extern "C" int sgfem_batch_solve(sgfem_batch* b, double rtol, int maxit, int check_every, double* x_out,
                                 sgfem_batch_stats* stats) {
    if (!b) return SGFEM_ERR_ARGUMENT;
    if (!b->finalized) return bfail(b, SGFEM_ERR_STATE, "batch not finalized");
    if (!(rtol > 0.0) || maxit <= 0) return bfail(b, SGFEM_ERR_ARGUMENT, "rtol must be > 0 and maxit > 0");
    check_every = std::max(1, std::min(check_every, 64));
    BCUDA(b, cudaSetDevice(b->device));
    const int B = (int)b->hp.size();
    const long long launches0 = b->launches;
    b->rtol = rtol;
    // right-hand sides (upload b0 of every problem, then build b, x = 0)
    std::vector<double> b0all;
    std::vector<long long> b0off(B);
    for (int i = 0; i < B; ++i) {
        b0off[i] = (long long)b0all.size();
        b0all.insert(b0all.end(), b->hp[i].b0.begin(), b->hp[i].b0.end());
    }
    double* d_b0 = nullptr;
    BCUDA(b, cudaMalloc((void**)&d_b0, b0all.size() * sizeof(double)));
    cudaError_t ce = cudaMemcpyAsync(d_b0, b0all.data(), b0all.size() * sizeof(double), cudaMemcpyHostToDevice, b->stream);
    std::vector<BProb> probs(B);
    if (ce == cudaSuccess)
        ce = cudaMemcpy(probs.data(), b->d_probs, (size_t)B * sizeof(BProb), cudaMemcpyDeviceToHost);
    if (ce != cudaSuccess) {
        cudaFree(d_b0);
        return bfail(b, SGFEM_ERR_CUDA, std::string("upload: ") + cudaGetErrorString(ce));
    }
    BCUDA(b, cudaEventRecord(b->ev0, b->stream));
    for (int i = 0; i < B; ++i) {
        const int g = (int)std::min<long long>(((long long)probs[i].n * probs[i].ld + 255) / 256, 1024);
        k_brhs<<<g, 256, 0, b->stream>>>(d_b0, b0off[i], b->d_b, b->d_x, probs[i].voff, probs[i].n, probs[i].ld,
                                         probs[i].bmask);
        BLAUNCHED(b);
    }
    int replays = 0;
    int status = SGFEM_OK;
    std::vector<int> iters(B, 0);
    std::vector<double> bb(B, 0.0), rr(B, 0.0);
    auto reset_scalars = [&](const std::vector<char>* active) {
        for (int i = 0; i < B; ++i) {
            KrylovScalars& s0 = b->h_scal[i];
            std::memset(&s0, 0, sizeof(s0));
            s0.first = 1;
            s0.done = (active && !(*active)[i]) ? 1 : 0;
        }
    };
    // per-problem squared norms of an FP64 vector (b or r) into h
    auto norms64 = [&](const double* v, std::vector<double>& h) -> int {
        for (auto& s0 : b->h_scal) std::memset(&s0, 0, sizeof(s0));
        BCUDA(b, cudaMemcpyAsync(b->d_scal, b->h_scal.data(), (size_t)B * sizeof(KrylovScalars), cudaMemcpyHostToDevice,
                                 b->stream));
        k_bjacobi<double><<<b->blocks, BT, 0, b->stream>>>(b->d_probs, b->d_bprob, v, nullptr, b->d_scal, b->d_part, 2);
        BLAUNCHED(b);
        k_bfin<<<B, BT, 0, b->stream>>>(b->d_probs, b->d_part, b->d_scal, BF_NORM, 0.0, maxit);
        BLAUNCHED(b);
        BCUDA(b, cudaMemcpyAsync(b->h_scal.data(), b->d_scal, (size_t)B * sizeof(KrylovScalars), cudaMemcpyDeviceToHost,
                                 b->stream));
        BCUDA(b, cudaStreamSynchronize(b->stream));
        for (int i = 0; i < B; ++i) h[i] = b->h_scal[i].rr;
        return SGFEM_OK;
    };
    const char* ep = getenv("SGFEM_BATCH_PRECISION");
    const bool fp64 = ep && std::string(ep) == "fp64";
    SG_TRY(norms64(b->d_b, bb));
    if (fp64) {
        // FP64 PCG on every problem
        BCUDA(b, cudaMemcpyAsync(b->d_r, b->d_b, (size_t)b->total * sizeof(double), cudaMemcpyDeviceToDevice, b->stream));
        reset_scalars(nullptr);
        const BVecs<double, double> v{b->d_x, b->d_r, b->d_p, b->d_q, b->d_z};
        SG_TRY((batch_pcg<double, double>(b, v, nullptr, rtol * rtol, maxit, check_every, &replays)));
        for (int i = 0; i < B; ++i) {
            iters[i] = b->h_scal[i].iters;
            rr[i] = b->h_scal[i].rr;
            if (b->h_scal[i].status != SGFEM_OK && status == SGFEM_OK) status = b->h_scal[i].status;
        }
    } else {
        // mixed: FP32 PCG on the correction of every unconverged problem, solution and
        // residual in FP64 (FP64 apply); first step to 1e-4, later steps aim to end the
        // solve (margin 3, at most a 1e-6 reduction per step)
        BCUDA(b, cudaMemcpyAsync(b->d_r, b->d_b, (size_t)b->total * sizeof(double), cudaMemcpyDeviceToDevice, b->stream));
        rr = bb;
        const BVecs<float, double> v{b->d_d64, b->d_r32, b->d_p32, b->d_q32, b->d_z32};
        std::vector<double> want(B, 0.0);
        for (int outer = 0; outer < 16; ++outer) {
            std::vector<char> active(B, 0);
            bool any = false;
            for (int i = 0; i < B; ++i) {
                active[i] = bb[i] > 0.0 && rr[i] > rtol * rtol * bb[i];
                any = any || active[i];
                const double finish = 0.1 * rtol * rtol * bb[i] / std::max(rr[i], 1e-300);
                want[i] = outer == 0 ? std::max(1e-8, finish) : std::max(finish, 1e-12);
            }
            if (!any) break;
            k_bdemote<<<b->blocks, BT, 0, b->stream>>>(b->d_probs, b->d_bprob, b->d_r, b->d_r32, b->d_d64, b->d_part);
            BLAUNCHED(b);
            BCUDA(b, cudaMemcpyAsync(b->d_want, want.data(), (size_t)B * sizeof(double), cudaMemcpyHostToDevice,
                                     b->stream));
            reset_scalars(&active);
            SG_TRY((batch_pcg<float, double>(b, v, b->d_want, 0.0, maxit, check_every, &replays)));
            for (int i = 0; i < B; ++i) {
                iters[i] += b->h_scal[i].iters;
                const int st0 = b->h_scal[i].status;
                if (st0 == SGFEM_ERR_BREAKDOWN || st0 == SGFEM_ERR_NONFINITE) status = st0;
            }
            if (status != SGFEM_OK) break;
            // x += d; r = b - A x (FP64)
            k_badd<<<b->blocks, BT, 0, b->stream>>>(b->d_probs, b->d_bprob, b->d_x, b->d_d64);
            BLAUNCHED(b);
            SG_TRY(apply64(b, b->d_x, b->d_q, b->d_part, nullptr));
            k_bresid<<<b->blocks, BT, 0, b->stream>>>(b->d_probs, b->d_bprob, b->d_b, b->d_q, b->d_r, b->d_part);
            BLAUNCHED(b);
            SG_TRY(norms64(b->d_r, rr));
            if (*std::max_element(iters.begin(), iters.end()) >= maxit) break;
        }
    }
    cudaFree(d_b0);
    cudaError_t ce2 = cudaSuccess;
    if (ce2 != cudaSuccess) return bfail(b, SGFEM_ERR_CUDA, std::string("batch iteration: ") + cudaGetErrorString(ce2));
    BCUDA(b, cudaEventRecord(b->ev1, b->stream));
    BCUDA(b, cudaEventSynchronize(b->ev1));
    float ms = 0.f;
    BCUDA(b, cudaEventElapsedTime(&ms, b->ev0, b->ev1));
    sgfem_batch_stats s{};
    s.time_ms = ms;
    s.graph_replays = replays;
    s.kernel_launches = b->launches - launches0;
    s.converged = 0;
    b->h_iters = iters;
    b->h_relres.assign(B, 0.0);
    for (int i = 0; i < B; ++i) {
        s.iterations_max = std::max(s.iterations_max, iters[i]);
        const double rel = bb[i] > 0.0 ? std::sqrt(rr[i] / bb[i]) : 0.0;
        b->h_relres[i] = rel;
        s.relres_max = std::max(s.relres_max, rel);
        if (rel <= rtol) s.converged++;
        else if (status == SGFEM_OK) status = SGFEM_ERR_MAXIT;
    }
    if (stats) *stats = s;
    if (x_out) {
        double* d_out = nullptr;
        long long ototal = 0;
        for (int i = 0; i < B; ++i) ototal += (long long)probs[i].n * probs[i].P;
        BCUDA(b, cudaMalloc((void**)&d_out, (size_t)ototal * sizeof(double)));
        long long oo = 0;
        for (int i = 0; i < B; ++i) {
            const int g = (int)std::min<long long>(((long long)probs[i].n * probs[i].P + 255) / 256, 1024);
            k_bout<<<g, 256, 0, b->stream>>>(b->d_x, probs[i].voff, probs[i].n, probs[i].ld, probs[i].P, d_out, oo);
            oo += (long long)probs[i].n * probs[i].P;
        }
        ce = cudaMemcpyAsync(x_out, d_out, (size_t)ototal * sizeof(double), cudaMemcpyDeviceToHost, b->stream);
        if (ce == cudaSuccess) ce = cudaStreamSynchronize(b->stream);
        cudaFree(d_out);
        if (ce != cudaSuccess) return bfail(b, SGFEM_ERR_CUDA, std::string("download: ") + cudaGetErrorString(ce));
    }
    if (status == SGFEM_ERR_MAXIT) return bfail(b, status, "some problems did not reach the tolerance within maxit");
    if (status != SGFEM_OK) return bfail(b, status, "a problem broke down (non-finite value or breakdown)");
    return SGFEM_OK;
}

extern "C" int sgfem_batch_problem_stats(const sgfem_batch* b, int i, int* iterations, double* relres) {
    if (!b || i < 0 || i >= (int)b->h_iters.size()) return SGFEM_ERR_ARGUMENT;
    if (iterations) *iterations = b->h_iters[i];
    if (relres) *relres = b->h_relres[i];
    return SGFEM_OK;
}
