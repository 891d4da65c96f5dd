// K5: evaluation of an SG solution at parameter samples and the sampling
// error integrals, on sm_103a.
//
// set_sample!(SGFEV, y[1:m]), src/sgfevector.jl:43-69 with
// src/tensorizedbasis.jl:226-252 and orthogonal_polynomials.jl:63-73:
//   u_m(y) = sum_k Psi_k(y) U[:, k],   Psi_k(y) = prod_{d<M} v_d[mu_k[d]],
//   v_d[j] = p_j(y_d) / ||p_j|| (d < m),  v_d = (1, 0, 0, ...) (d >= m).
// calculate_sampling_error, src/sampling_error.jl:2-44 and :149-191:
//   errH1[m, s] = sum_T int_T |grad(u_s - u_m(y_s))|^2,
//   errL2[m, s] = sum_T int_T (u_s - u_m(y_s))^2,            m = 0..M.
//
// Kernels
//   k_psi            one thread per (mode, sample): Psi by the three-term
//                    recurrence, with the rounding steps of the host code
//                    (no contraction), so Psi is bitwise the host value.
//   k_eval_gemm      out = U Psi (n x P times P x S), 64 x 64 output tiles
//                    staged through shared memory, FP64 FMA.
//   k_sampling_error one warp per (group of cells, 32 samples), lane = sample.
//                    Per cell the warp evaluates the deterministic solution
//                    at the quadrature points once, then walks the SG modes
//                    sorted by their last active dimension sup(mu_k): after the
//                    modes with sup = m the running local coefficients are the
//                    SG solution truncated to y[1:m], so every truncation level
//                    costs one quadrature pass and no mode is visited twice.
//                    Per-lane sums over the warp's cells go to per-group
//                    partials that a second kernel adds in group order, so the
//                    result is bitwise reproducible.  FP64 throughout.
#include <algorithm>
#include <array>
#include <cmath>
#include <numeric>
#include <string>
#include <vector>

#include "fe_basis.cuh"
#include "sgfem_internal.h"

namespace {

constexpr int SW = 4;  // warps per block of k_sampling_error

__global__ void k_psi(int P, int M, int S, const int* __restrict__ mi, const double* __restrict__ rec,
                      const double* __restrict__ norms, const double* __restrict__ y, int ys, int yoff, int mtrunc,
                      double* __restrict__ psi, int lds) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (int64_t)P * S) return;
    const int k = (int)(t / S), s = (int)(t % S);
    double v = 1.0;
    for (int d = 0; d < M; ++d) {
        const int j = mi[(size_t)k * M + d];
        if (d >= mtrunc) {
            if (j != 0) {
                v = 0.0;
                break;
            }
            continue;
        }
        const double x = y[(size_t)s * ys + yoff + d];
        double pm = 0.0, p = 1.0;
        for (int i = 0; i < j; ++i) {
            double pn = __dmul_rn(__dadd_rn(rec[3 * i], __dmul_rn(rec[3 * i + 1], x)), p);
            if (i > 0) pn = __dsub_rn(pn, __dmul_rn(rec[3 * i + 2], pm));
            pm = p;
            p = pn;
        }
        v = __dmul_rn(v, __ddiv_rn(p, norms[j]));
    }
    psi[(size_t)k * lds + s] = v;
}

// out[s * n + i] = sum_k U[k * n + i] psi[k * lds + s]
__global__ void __launch_bounds__(256) k_eval_gemm(const double* __restrict__ U, const double* __restrict__ psi, int n,
                                                   int P, int S, int lds, double* __restrict__ out) {
    __shared__ double As[16][64];
    __shared__ double Bs[16][64];
    const int i0 = blockIdx.x * 64, s0 = blockIdx.y * 64;
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    double acc[4][4];
#pragma unroll
    for (int r = 0; r < 4; ++r)
#pragma unroll
        for (int c = 0; c < 4; ++c) acc[r][c] = 0.0;
    for (int k0 = 0; k0 < P; k0 += 16) {
        for (int l = threadIdx.x; l < 1024; l += 256) {
            const int kk = l >> 6, ii = l & 63, k = k0 + kk;
            As[kk][ii] = (k < P && i0 + ii < n) ? U[(size_t)k * n + i0 + ii] : 0.0;
            Bs[kk][ii] = (k < P && s0 + ii < S) ? psi[(size_t)k * lds + s0 + ii] : 0.0;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < 16; ++kk) {
            double a[4], b[4];
#pragma unroll
            for (int r = 0; r < 4; ++r) a[r] = As[kk][tx + 16 * r];
#pragma unroll
            for (int c = 0; c < 4; ++c) b[c] = Bs[kk][ty + 16 * c];
#pragma unroll
            for (int r = 0; r < 4; ++r)
#pragma unroll
                for (int c = 0; c < 4; ++c) acc[r][c] = fma(a[r], b[c], acc[r][c]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        const int s = s0 + ty + 16 * c;
        if (s >= S) continue;
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            const int i = i0 + tx + 16 * r;
            if (i < n) out[(size_t)s * n + i] = acc[r][c];
        }
    }
}

struct SCell {
    double g[6];  // grad lambda_0..2
    double vol;
};

struct ErrArgs {
    int od, os, nq, ncells, S, ld, M, nsg, groups, lds;
    const SCell* cg;
    const int* ddofs;    // NDD per cell: device rows of D
    const int* sdofs;    // NDS per cell: SG dofs
    const double* D;     // deterministic solutions, device layout (n_det rows x ld)
    const double* U;     // P x nsg, modes sorted by sup
    const double* psi;   // P x lds, same order
    const int* kptr;     // M + 2: modes with sup = m are [kptr[m], kptr[m+1])
    const double* xq;    // 2 x nq
    const double* wq;    // nq, sum 1
    double* part;        // groups x (M+1) x 2 x S
};

template <int NDD, int NDS>
__global__ void __launch_bounds__(SW * 32) k_sampling_error(ErrArgs a) {
    extern __shared__ double ssm[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int nq = a.nq;
    double* phiD = ssm;                 // nq x NDD reference values
    double* phiS = phiD + nq * NDD;     // nq x NDS
    double* w = phiS + nq * NDS;        // nq
    const int per_warp = nq * 2 * (NDD + NDS) + nq * 3 * 32 + (a.M + 1) * 2 * 32;
    double* gD = w + nq + (size_t)warp * per_warp;  // [q][i][2] physical gradients
    double* gS = gD + nq * NDD * 2;
    double* ud = gS + nq * NDS * 2;                 // [q][3][32]: u, du/dx, du/dy of the lane's sample
    double* acc = ud + nq * 3 * 32;                 // [m][2][32]
    for (int q = threadIdx.x; q < nq; q += blockDim.x) {
        const double lam[3] = {1.0 - a.xq[2 * q] - a.xq[2 * q + 1], a.xq[2 * q], a.xq[2 * q + 1]};
        double v[6];
        sgfem_fe::basis_val(a.od, lam, v);
        for (int i = 0; i < NDD; ++i) phiD[q * NDD + i] = v[i];
        sgfem_fe::basis_val(a.os, lam, v);
        for (int i = 0; i < NDS; ++i) phiS[q * NDS + i] = v[i];
        w[q] = a.wq[q];
    }
    for (int t = 0; t <= a.M; ++t) {
        acc[(2 * t) * 32 + lane] = 0.0;
        acc[(2 * t + 1) * 32 + lane] = 0.0;
    }
    __syncthreads();
    const int chunks = (a.S + 31) / 32;
    const int wid = blockIdx.x * SW + warp;
    const int chunk = wid % chunks, group = wid / chunks;
    if (group >= a.groups) return;
    const int s = chunk * 32 + lane;
    const bool live = s < a.S;
    for (int c = group; c < a.ncells; c += a.groups) {
        const SCell G = a.cg[c];
        __syncwarp();
        for (int q = lane; q < nq; q += 32) {
            const double lam[3] = {1.0 - a.xq[2 * q] - a.xq[2 * q + 1], a.xq[2 * q], a.xq[2 * q + 1]};
            double gg[12];
            sgfem_fe::basis_grad(a.od, G.g, lam, gg);
            for (int i = 0; i < 2 * NDD; ++i) gD[q * NDD * 2 + i] = gg[i];
            sgfem_fe::basis_grad(a.os, G.g, lam, gg);
            for (int i = 0; i < 2 * NDS; ++i) gS[q * NDS * 2 + i] = gg[i];
        }
        __syncwarp();
        double dv[NDD];
#pragma unroll
        for (int i = 0; i < NDD; ++i) dv[i] = live ? a.D[(size_t)a.ddofs[(size_t)c * NDD + i] * a.ld + s] : 0.0;
        for (int q = 0; q < nq; ++q) {
            double u = 0.0, ux = 0.0, uy = 0.0;
#pragma unroll
            for (int i = 0; i < NDD; ++i) {
                u = fma(dv[i], phiD[q * NDD + i], u);
                ux = fma(dv[i], gD[(q * NDD + i) * 2], ux);
                uy = fma(dv[i], gD[(q * NDD + i) * 2 + 1], uy);
            }
            ud[(q * 3) * 32 + lane] = u;
            ud[(q * 3 + 1) * 32 + lane] = ux;
            ud[(q * 3 + 2) * 32 + lane] = uy;
        }
        int sd[NDS];
        double us[NDS];
#pragma unroll
        for (int i = 0; i < NDS; ++i) {
            sd[i] = a.sdofs[(size_t)c * NDS + i];
            us[i] = 0.0;
        }
        for (int m = 0; m <= a.M; ++m) {
            const int k1 = a.kptr[m + 1];
            for (int k = a.kptr[m]; k < k1; ++k) {
                const double ps = live ? a.psi[(size_t)k * a.lds + s] : 0.0;
                const double* Uk = a.U + (size_t)k * a.nsg;
#pragma unroll
                for (int i = 0; i < NDS; ++i) us[i] = fma(__ldg(Uk + sd[i]), ps, us[i]);
            }
            double eh = 0.0, el = 0.0;
            for (int q = 0; q < nq; ++q) {
                double e = ud[(q * 3) * 32 + lane], ex = ud[(q * 3 + 1) * 32 + lane], ey = ud[(q * 3 + 2) * 32 + lane];
#pragma unroll
                for (int i = 0; i < NDS; ++i) {
                    e = fma(-us[i], phiS[q * NDS + i], e);
                    ex = fma(-us[i], gS[(q * NDS + i) * 2], ex);
                    ey = fma(-us[i], gS[(q * NDS + i) * 2 + 1], ey);
                }
                eh = fma(w[q], ex * ex + ey * ey, eh);
                el = fma(w[q], e * e, el);
            }
            acc[(2 * m) * 32 + lane] += G.vol * eh;
            acc[(2 * m + 1) * 32 + lane] += G.vol * el;
        }
    }
    if (live) {
        double* out = a.part + (size_t)group * (a.M + 1) * 2 * a.S;
        for (int m = 0; m <= a.M; ++m) {
            out[(size_t)(2 * m) * a.S + s] = acc[(2 * m) * 32 + lane];
            out[(size_t)(2 * m + 1) * a.S + s] = acc[(2 * m + 1) * 32 + lane];
        }
    }
}

// The same sums as quadratic forms, where the SG space embeds in the deterministic one
// (P1 in P2, equal orders): psi_j = sum_i E_ij phi_i with E_ij = psi_j(node_i), so on
// every cell e = u_s - u_sg,m = sum_i c_i phi_i with c = d - E us, and with matrices
// built from the caller's rule
//   sum_q w_q e(x_q)^2        = c' Mq c,     Mq_ij  = sum_q w_q phi_i phi_j,
//   sum_q w_q |grad e(x_q)|^2 = c' K_T c,    K_T_ij = sum_{k,l} (g_k . g_l) R^kl_ij,
//   R^kl_ij = sum_q w_q (dphi_i/dlam_k)(dphi_j/dlam_l),
// the quadrature sums of k_sampling_error up to rounding, for any rule.  K_T
// annihilates constants, so the gradient form takes c_i - c_0 (a nearly constant error
// does not cancel).  Per (cell, sample, level): NDD NDS + ~2 NDD^2 FMAs instead of
// nq (3 NDS + 4), and no quadrature pass over u_s per cell.
__host__ __device__ constexpr int ut_index(int i, int j, int n) { return i * n - i * (i - 1) / 2 + (j - i); }

struct QfArgs {
    int ncells, S, ld, M, nsg, groups, lds;
    const double* vol;   // ncells
    const double* KT;    // ncells x NDD(NDD+1)/2, upper triangle row by row
    const double* E;     // NDD x NDS
    const double* Mq;    // NDD(NDD+1)/2
    const int* ddofs;
    const int* sdofs;
    const double* D;
    const double* U;
    const double* psi;
    const int* kptr;
    double* part;
};

template <int NDD, int NDS>
__global__ void __launch_bounds__(SW * 32) k_sampling_error_qf(QfArgs a) {
    constexpr int NT = NDD * (NDD + 1) / 2;
    extern __shared__ double ssm[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    double* sE = ssm;                                          // NDD x NDS
    double* sM = sE + NDD * NDS;                               // NT
    double* acc = sM + NT + (size_t)warp * (a.M + 1) * 2 * 32;  // [m][2][32]
    for (int t = threadIdx.x; t < NDD * NDS; t += blockDim.x) sE[t] = a.E[t];
    for (int t = threadIdx.x; t < NT; t += blockDim.x) sM[t] = a.Mq[t];
    for (int t = 0; t <= a.M; ++t) {
        acc[(2 * t) * 32 + lane] = 0.0;
        acc[(2 * t + 1) * 32 + lane] = 0.0;
    }
    __syncthreads();
    const int chunks = (a.S + 31) / 32;
    const int wid = blockIdx.x * SW + warp;
    const int chunk = wid % chunks, group = wid / chunks;
    if (group >= a.groups) return;
    const int s = chunk * 32 + lane;
    const bool live = s < a.S;
    for (int c = group; c < a.ncells; c += a.groups) {
        double K[NT];
#pragma unroll
        for (int t = 0; t < NT; ++t) K[t] = __ldg(a.KT + (size_t)c * NT + t);
        const double vol = __ldg(a.vol + c);
        double d[NDD];
#pragma unroll
        for (int i = 0; i < NDD; ++i) d[i] = live ? a.D[(size_t)a.ddofs[(size_t)c * NDD + i] * a.ld + s] : 0.0;
        int sd[NDS];
        double us[NDS];
#pragma unroll
        for (int i = 0; i < NDS; ++i) {
            sd[i] = a.sdofs[(size_t)c * NDS + i];
            us[i] = 0.0;
        }
        for (int m = 0; m <= a.M; ++m) {
            const int k1 = a.kptr[m + 1];
            for (int k = a.kptr[m]; k < k1; ++k) {
                const double ps = live ? a.psi[(size_t)k * a.lds + s] : 0.0;
                const double* Uk = a.U + (size_t)k * a.nsg;
#pragma unroll
                for (int i = 0; i < NDS; ++i) us[i] = fma(__ldg(Uk + sd[i]), ps, us[i]);
            }
            double e[NDD];
#pragma unroll
            for (int i = 0; i < NDD; ++i) {
                double v = d[i];
#pragma unroll
                for (int j = 0; j < NDS; ++j) v = fma(-sE[i * NDS + j], us[j], v);
                e[i] = v;
            }
            double el = 0.0;
#pragma unroll
            for (int i = 0; i < NDD; ++i) {
                double off = 0.0;
#pragma unroll
                for (int j = i + 1; j < NDD; ++j) off = fma(sM[ut_index(i, j, NDD)], e[j], off);
                el = fma(e[i], fma(2.0, off, sM[ut_index(i, i, NDD)] * e[i]), el);
            }
            double f[NDD];
#pragma unroll
            for (int i = 1; i < NDD; ++i) f[i] = e[i] - e[0];
            double eh = 0.0;
#pragma unroll
            for (int i = 1; i < NDD; ++i) {
                double off = 0.0;
#pragma unroll
                for (int j = i + 1; j < NDD; ++j) off = fma(K[ut_index(i, j, NDD)], f[j], off);
                eh = fma(f[i], fma(2.0, off, K[ut_index(i, i, NDD)] * f[i]), eh);
            }
            acc[(2 * m) * 32 + lane] += vol * eh;
            acc[(2 * m + 1) * 32 + lane] += vol * el;
        }
    }
    if (live) {
        double* out = a.part + (size_t)group * (a.M + 1) * 2 * a.S;
        for (int m = 0; m <= a.M; ++m) {
            out[(size_t)(2 * m) * a.S + s] = acc[(2 * m) * 32 + lane];
            out[(size_t)(2 * m + 1) * a.S + s] = acc[(2 * m + 1) * 32 + lane];
        }
    }
}

// errH1/errL2[s * (M+1) + m] = sum over groups in order
__global__ void k_sampling_reduce(const double* __restrict__ part, int groups, int M, int S, double* __restrict__ eh,
                                  double* __restrict__ el) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int per = (M + 1) * 2 * S;
    if (t >= per) return;
    double v = 0.0;
    for (int g = 0; g < groups; ++g) v += part[(size_t)g * per + t];
    const int s = t % S, mh = t / S, m = mh >> 1;
    ((mh & 1) ? el : eh)[(size_t)s * (M + 1) + m] = v;
}

// The arrays of one call packed at 256-byte offsets into a context buffer that only
// grows: no cudaMalloc / cudaFree (which synchronises the device) per call.  Host
// sources stay alive until the call's final stream synchronisation.
struct Pack {
    struct Item {
        const void* src;  // nullptr: scratch
        size_t bytes;
        void** dst;
    };
    std::vector<Item> items;
    template <typename T>
    void up(const T* src, size_t n, T** dst) {
        items.push_back({src, n * sizeof(T), (void**)dst});
    }
    template <typename T>
    void scratch(size_t n, T** dst) {
        items.push_back({nullptr, n * sizeof(T), (void**)dst});
    }
    static size_t pad(size_t b) { return (std::max<size_t>(b, 1) + 255) / 256 * 256; }
    int commit(sgfem_context* ctx, DeviceBuf& buf) {
        size_t total = 0;
        for (const Item& it : items) total += pad(it.bytes);
        SG_TRY(sg_ensure(ctx, buf, total));
        size_t off = 0;
        for (const Item& it : items) {
            *it.dst = (char*)buf.p + off;
            if (it.src && it.bytes)
                SG_CUDA(ctx, cudaMemcpyAsync(*it.dst, it.src, it.bytes, cudaMemcpyHostToDevice, ctx->stream));
            off += pad(it.bytes);
        }
        return SGFEM_OK;
    }
};

// checks of the basis description; sup[k] = last dimension (1-based) with mu_k[d] > 0
int check_basis(sgfem_context* ctx, const sgfem_sg_basis* b, std::vector<int>& sup) {
    if (b->P <= 0 || b->M < 0 || b->M > 4095 || b->P > (1 << 24) || b->maxorder < 0 || b->maxorder > 64)
        return sg_fail(ctx, SGFEM_ERR_ARGUMENT, "sg basis: bad sizes");
    if ((b->M > 0 && !b->multi_indices) || !b->norms || (b->maxorder > 0 && !b->recurrence))
        return sg_fail(ctx, SGFEM_ERR_ARGUMENT, "sg basis: null pointer");
    sup.assign(b->P, 0);
    for (int64_t k = 0; k < b->P; ++k)
        for (int64_t d = 0; d < b->M; ++d) {
            const int j = b->multi_indices[k * b->M + d];
            if (j < 0 || j > b->maxorder) return sg_fail(ctx, SGFEM_ERR_ARGUMENT, "multi-index entry outside 0..maxorder");
            if (j > 0) sup[k] = (int)d + 1;
        }
    for (int j = 0; j <= b->maxorder; ++j)
        if (!(b->norms[j] > 0.0) || !std::isfinite(b->norms[j])) return sg_fail(ctx, SGFEM_ERR_ARGUMENT, "norms must be positive");
    return SGFEM_OK;
}

int launch_psi(sgfem_context* ctx, const sgfem_sg_basis* b, const int* d_mi, const double* d_rec, const double* d_norms,
               const double* d_y, int ys, int yoff, int mtrunc, int S, double* d_psi, int lds) {
    const int64_t total = b->P * (int64_t)S;
    const int blocks = (int)((total + 255) / 256);
    k_psi<<<blocks, 256, 0, ctx->stream>>>((int)b->P, (int)b->M, S, d_mi, d_rec, d_norms, d_y, ys, yoff, mtrunc, d_psi,
                                          lds);
    SG_LAUNCHED(ctx);
    return SGFEM_OK;
}

// d phi_i / d lam_k (k = 0..2) of the P1 / P2 basis at barycentric lam, out[i * 3 + k]
void basis_dlam(int order, const double* lam, double* out) {
    std::fill(out, out + 18, 0.0);
    if (order == 1) {
        for (int i = 0; i < 3; ++i) out[i * 3 + i] = 1.0;
        return;
    }
    const int ea[3] = {0, 1, 2}, eb[3] = {1, 2, 0};
    for (int i = 0; i < 3; ++i) out[i * 3 + i] = 4.0 * lam[i] - 1.0;
    for (int e = 0; e < 3; ++e) {
        out[(3 + e) * 3 + ea[e]] = 4.0 * lam[eb[e]];
        out[(3 + e) * 3 + eb[e]] = 4.0 * lam[ea[e]];
    }
}

// Quadratic-form data of k_sampling_error_qf from the cell rule: E (SG basis in the
// deterministic one, false when it does not embed), Mq and the six symmetric
// combinations Rs[(k,l), k <= l] of R^kl (R^kl + R^lk off the diagonal).
bool quadform_tables(int od, int os, int nq, const double* xq, const double* wq, std::vector<double>& E,
                     std::vector<double>& Mq, std::vector<double>& Rs) {
    const int ndd = sgfem_fe::ndofs4cell(od), nds = sgfem_fe::ndofs4cell(os), nt = ndd * (ndd + 1) / 2;
    // nodes of the deterministic basis: vertices, then the midpoints of (0,1), (1,2), (2,0)
    const double nodes[6][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}, {0.5, 0.5, 0}, {0, 0.5, 0.5}, {0.5, 0, 0.5}};
    E.assign((size_t)ndd * nds, 0.0);
    double v[6], w6[6];
    for (int i = 0; i < ndd; ++i) {
        sgfem_fe::basis_val(os, nodes[i], v);
        for (int j = 0; j < nds; ++j) E[(size_t)i * nds + j] = v[j];
    }
    // the embedding holds where sum_i E_ij phi_i = psi_j on a set that determines quadratics
    std::vector<std::array<double, 3>> pts;
    for (int q = 0; q < nq; ++q) pts.push_back({1.0 - xq[2 * q] - xq[2 * q + 1], xq[2 * q], xq[2 * q + 1]});
    for (auto& nd : nodes) pts.push_back({nd[0], nd[1], nd[2]});
    pts.push_back({1.0 / 3, 1.0 / 3, 1.0 / 3});
    pts.push_back({0.2, 0.3, 0.5});
    pts.push_back({0.6, 0.1, 0.3});
    for (auto& lam : pts) {
        sgfem_fe::basis_val(od, lam.data(), w6);
        sgfem_fe::basis_val(os, lam.data(), v);
        for (int j = 0; j < nds; ++j) {
            double t = 0.0;
            for (int i = 0; i < ndd; ++i) t += E[(size_t)i * nds + j] * w6[i];
            if (std::fabs(t - v[j]) > 1e-13) return false;
        }
    }
    Mq.assign(nt, 0.0);
    Rs.assign((size_t)6 * nt, 0.0);
    const int kk[6] = {0, 1, 2, 0, 0, 1}, ll[6] = {0, 1, 2, 1, 2, 2};
    double dl[18];
    for (int q = 0; q < nq; ++q) {
        const double lam[3] = {1.0 - xq[2 * q] - xq[2 * q + 1], xq[2 * q], xq[2 * q + 1]};
        sgfem_fe::basis_val(od, lam, w6);
        basis_dlam(od, lam, dl);
        for (int i = 0; i < ndd; ++i)
            for (int j = i; j < ndd; ++j) {
                const int t = ut_index(i, j, ndd);
                Mq[t] += wq[q] * w6[i] * w6[j];
                for (int r = 0; r < 6; ++r) {
                    const int k = kk[r], l = ll[r];
                    double g = dl[i * 3 + k] * dl[j * 3 + l];
                    if (k != l) g += dl[i * 3 + l] * dl[j * 3 + k];
                    Rs[(size_t)r * nt + t] += wq[q] * g;
                }
            }
    }
    return true;
}

template <int NDD, int NDS>
int launch_error_qf(sgfem_context* ctx, const QfArgs& a, int blocks, size_t smem) {
    if (smem > 48 * 1024)
        SG_CUDA(ctx, cudaFuncSetAttribute(k_sampling_error_qf<NDD, NDS>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)smem));
    k_sampling_error_qf<NDD, NDS><<<blocks, SW * 32, smem, ctx->stream>>>(a);
    SG_LAUNCHED(ctx);
    return SGFEM_OK;
}

template <int NDD, int NDS>
int launch_error(sgfem_context* ctx, const ErrArgs& a, int blocks, size_t smem) {
    if (smem > 48 * 1024)
        SG_CUDA(ctx, cudaFuncSetAttribute(k_sampling_error<NDD, NDS>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)smem));
    k_sampling_error<NDD, NDS><<<blocks, SW * 32, smem, ctx->stream>>>(a);
    SG_LAUNCHED(ctx);
    return SGFEM_OK;
}

}  // namespace

extern "C" int sgfem_evaluate_samples(sgfem_context* ctx, const double* U, int64_t n, const sgfem_sg_basis* basis,
                                      const double* y, int64_t Ms, int64_t S, int64_t m, double* out) {
    SG_TRY(sg_check_ready(ctx));
    if (!U || !basis || !out || (Ms > 0 && !y)) return sg_fail(ctx, SGFEM_ERR_ARGUMENT, "sgfem_evaluate_samples: null argument");
    if (n <= 0 || n > INT32_MAX || S <= 0 || S > (1 << 24) || Ms < 0 || m < 0 || m > Ms)
        return sg_fail(ctx, SGFEM_ERR_ARGUMENT, "sgfem_evaluate_samples: bad sizes (need 0 <= m <= Ms)");
    std::vector<int> sup;
    SG_TRY(check_basis(ctx, basis, sup));
    for (int64_t t = 0; t < Ms * S; ++t)
        if (!std::isfinite(y[t])) return sg_fail(ctx, SGFEM_ERR_NONFINITE, "non-finite sample");
    SG_CUDA(ctx, cudaSetDevice(ctx->device));
    Pack pk;
    const int lds = (int)((S + 31) / 32 * 32);
    std::vector<int> mi(basis->multi_indices, basis->multi_indices + basis->P * basis->M);
    int* d_mi;
    double *d_rec, *d_norms, *d_y, *d_U, *d_psi, *d_out;
    pk.up(mi.data(), mi.size(), &d_mi);
    pk.up(basis->recurrence, (size_t)3 * basis->maxorder, &d_rec);
    pk.up(basis->norms, (size_t)basis->maxorder + 1, &d_norms);
    pk.up(y, (size_t)(Ms * S), &d_y);
    pk.up(U, (size_t)(n * basis->P), &d_U);
    pk.scratch((size_t)basis->P * lds, &d_psi);
    pk.scratch((size_t)(n * S), &d_out);
    SG_TRY(pk.commit(ctx, ctx->w_samp));
    // dimensions beyond Ms count as truncated: m <= Ms, so d < m only reads stored dimensions
    SG_TRY(launch_psi(ctx, basis, d_mi, d_rec, d_norms, d_y, (int)Ms, 0, (int)m, (int)S, d_psi, lds));
    dim3 grid((unsigned)((n + 63) / 64), (unsigned)((S + 63) / 64));
    k_eval_gemm<<<grid, 256, 0, ctx->stream>>>(d_U, d_psi, (int)n, (int)basis->P, (int)S, lds, d_out);
    SG_LAUNCHED(ctx);
    SG_CUDA(ctx, cudaMemcpyAsync(out, d_out, (size_t)(n * S) * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    SG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return SGFEM_OK;
}

extern "C" int sgfem_sampling_error(sgfem_context* ctx, const double* det_solutions, const sgfem_mesh* mesh,
                                    const sgfem_fe_space* sg_space, const double* U, const sgfem_sg_basis* basis,
                                    const sgfem_quadrature* quad, double* errH1, double* errL2) {
    SG_TRY(sg_check_ready(ctx));
    if (!ctx->batched) return sg_fail(ctx, SGFEM_ERR_STATE, "sgfem_sampling_error needs a samples context (sgfem_set_samples)");
    if (!mesh || !sg_space || !U || !basis || !quad || !errH1 || !errL2)
        return sg_fail(ctx, SGFEM_ERR_ARGUMENT, "sgfem_sampling_error: null argument");
    if ((mesh->order != 1 && mesh->order != 2) || (sg_space->order != 1 && sg_space->order != 2))
        return sg_fail(ctx, SGFEM_ERR_ARGUMENT, "orders must be 1 or 2");
    if (!mesh->coords || !mesh->cell_nodes || !mesh->cell_dofs || !mesh->cell_volumes || !sg_space->cell_dofs)
        return sg_fail(ctx, SGFEM_ERR_ARGUMENT, "sgfem_sampling_error: null mesh array");
    const int ndd = sgfem_fe::ndofs4cell(mesh->order), nds = sgfem_fe::ndofs4cell(sg_space->order);
    const int64_t nc = mesh->ncells, nn = mesh->nnodes, nsg = sg_space->ndofs;
    const int nq = quad->nq;
    if (nc <= 0 || nc > INT32_MAX || nn <= 0 || nsg <= 0 || nsg > INT32_MAX || nq <= 0 || nq > 64 || !quad->xref || !quad->w)
        return sg_fail(ctx, SGFEM_ERR_ARGUMENT, "empty mesh, space or quadrature (nq <= 64)");
    std::vector<int> sup;
    SG_TRY(check_basis(ctx, basis, sup));
    const int64_t S = ctx->P, P = basis->P, M = basis->M;
    if (M > ctx->M)
        return sg_fail(ctx, SGFEM_ERR_ARGUMENT, "multi-indices longer than the sample dimension of the context");
    SG_CUDA(ctx, cudaSetDevice(ctx->device));

    // deterministic solutions
    const size_t n64 = sg_vec_bytes(ctx, SGFEM_FP64);
    if (det_solutions) {
        SG_TRY(sg_ensure(ctx, ctx->w_vec[10], n64));
        SG_TRY(sgfem_to_device_layout(ctx, det_solutions, ctx->w_vec[10].p, SGFEM_FP64));
        ctx->samples_x_valid = true;
    } else if (!ctx->samples_x_valid) {
        return sg_fail(ctx, SGFEM_ERR_STATE, "no device-resident solutions of the current samples (run sgfem_solve_samples)");
    }

    // geometry and dof maps
    std::vector<SCell> cg(nc);
    std::vector<int> ddofs((size_t)nc * ndd), sdofs((size_t)nc * nds);
    for (int64_t c = 0; c < nc; ++c) {
        const int64_t* cn = mesh->cell_nodes + 3 * c;
        double px[3], py[3];
        for (int k = 0; k < 3; ++k) {
            const int64_t v = cn[k] - 1;
            if (v < 0 || v >= nn) return sg_fail(ctx, SGFEM_ERR_ARGUMENT, "cell_nodes out of range");
            px[k] = mesh->coords[2 * v];
            py[k] = mesh->coords[2 * v + 1];
        }
        const double j00 = px[1] - px[0], j01 = px[2] - px[0], j10 = py[1] - py[0], j11 = py[2] - py[0];
        const double det = j00 * j11 - j01 * j10;
        if (det == 0.0) return sg_fail(ctx, SGFEM_ERR_ARGUMENT, "degenerate cell");
        SCell& G = cg[c];
        const double i00 = j11 / det, i01 = -j01 / det, i10 = -j10 / det, i11 = j00 / det;
        G.g[2] = i00; G.g[3] = i01;
        G.g[4] = i10; G.g[5] = i11;
        G.g[0] = -i00 - i10; G.g[1] = -i01 - i11;
        G.vol = mesh->cell_volumes[c];
        for (int d = 0; d < ndd; ++d) {
            const int64_t dof = mesh->cell_dofs[(size_t)ndd * c + d] - 1;
            if (dof < 0 || dof >= ctx->n) return sg_fail(ctx, SGFEM_ERR_ARGUMENT, "deterministic cell_dofs out of range");
            ddofs[(size_t)c * ndd + d] = ctx->iperm[dof];
        }
        for (int d = 0; d < nds; ++d) {
            const int64_t dof = sg_space->cell_dofs[(size_t)nds * c + d] - 1;
            if (dof < 0 || dof >= nsg) return sg_fail(ctx, SGFEM_ERR_ARGUMENT, "SG cell_dofs out of range");
            sdofs[(size_t)c * nds + d] = (int)dof;
        }
    }

    // modes sorted by sup (stable), their multi-indices and U columns in that order
    std::vector<int> order(P);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int x, int z) { return sup[x] < sup[z]; });
    std::vector<int> kptr(M + 2, 0);
    for (int64_t k = 0; k < P; ++k) kptr[sup[k] + 1]++;
    for (int64_t m = 0; m <= M; ++m) kptr[m + 1] += kptr[m];
    std::vector<int> mi((size_t)P * M);
    std::vector<double> Us((size_t)P * nsg);
    for (int64_t kk = 0; kk < P; ++kk) {
        const int k = order[kk];
        for (int64_t d = 0; d < M; ++d) mi[(size_t)kk * M + d] = basis->multi_indices[(size_t)k * M + d];
        std::copy(U + (size_t)k * nsg, U + (size_t)(k + 1) * nsg, Us.begin() + (size_t)kk * nsg);
    }
    sgfem_sg_basis sorted = *basis;
    sorted.multi_indices = mi.data();

    const int lds = (int)((S + 31) / 32 * 32);
    const int chunks = (int)((S + 31) / 32);
    const int target = std::max(1, ctx->num_sms) * 16;
    const int groups = (int)std::max<int64_t>(1, std::min<int64_t>(nc, (target + chunks - 1) / chunks));
    const int64_t warps = (int64_t)groups * chunks;
    const int blocks = (int)((warps + SW - 1) / SW);
    const size_t per = (size_t)(M + 1) * 2 * S;
    // quadratic forms where the SG space embeds in the deterministic one (SGFEM_SAMPLING_QF=0:
    // the quadrature kernel always)
    std::vector<double> E, Mq, Rs;
    const char* eqf = getenv("SGFEM_SAMPLING_QF");
    bool qf = !(eqf && atoi(eqf) == 0) && quadform_tables(mesh->order, sg_space->order, nq, quad->xref, quad->w, E, Mq, Rs);
    const size_t smem_qf = sizeof(double) * ((size_t)ndd * nds + Mq.size() + (size_t)SW * (M + 1) * 2 * 32);
    qf = qf && smem_qf <= 227 * 1024;
    const size_t smem = sizeof(double) * ((size_t)nq * (ndd + nds + 1) +
                                          (size_t)SW * (nq * 2 * (ndd + nds) + nq * 3 * 32 + (M + 1) * 2 * 32));
    if (!qf && smem > 227 * 1024)
        return sg_fail(ctx, SGFEM_ERR_UNSUPPORTED,
                       "sampling error: too many truncation levels or quadrature points for shared memory");
    const int nt = ndd * (ndd + 1) / 2;
    std::vector<double> KT, vol;
    if (qf) {
        const int kk[6] = {0, 1, 2, 0, 0, 1}, ll[6] = {0, 1, 2, 1, 2, 2};
        KT.resize((size_t)nc * nt);
        vol.resize(nc);
        for (int64_t c = 0; c < nc; ++c) {
            const double* g = cg[c].g;
            double G[6];
            for (int r = 0; r < 6; ++r) G[r] = g[2 * kk[r]] * g[2 * ll[r]] + g[2 * kk[r] + 1] * g[2 * ll[r] + 1];
            for (int t = 0; t < nt; ++t) {
                double v = 0.0;
                for (int r = 0; r < 6; ++r) v += G[r] * Rs[(size_t)r * nt + t];
                KT[(size_t)c * nt + t] = v;
            }
            vol[c] = cg[c].vol;
        }
    }

    Pack pk;
    int *d_mi, *d_kptr, *d_dd, *d_sd;
    double *d_rec, *d_norms, *d_U, *d_psi, *d_xq, *d_wq, *d_part, *d_eh, *d_el;
    double *d_KT = nullptr, *d_vol = nullptr, *d_E = nullptr, *d_Mq = nullptr;
    SCell* d_cg;
    pk.up(mi.data(), mi.size(), &d_mi);
    pk.up(basis->recurrence, (size_t)3 * basis->maxorder, &d_rec);
    pk.up(basis->norms, (size_t)basis->maxorder + 1, &d_norms);
    pk.up(Us.data(), Us.size(), &d_U);
    pk.up(kptr.data(), kptr.size(), &d_kptr);
    pk.up(ddofs.data(), ddofs.size(), &d_dd);
    pk.up(sdofs.data(), sdofs.size(), &d_sd);
    pk.scratch((size_t)P * lds, &d_psi);
    pk.scratch(per * groups, &d_part);
    pk.scratch((size_t)(M + 1) * S, &d_eh);
    pk.scratch((size_t)(M + 1) * S, &d_el);
    if (qf) {
        pk.up(KT.data(), KT.size(), &d_KT);
        pk.up(vol.data(), vol.size(), &d_vol);
        pk.up(E.data(), E.size(), &d_E);
        pk.up(Mq.data(), Mq.size(), &d_Mq);
    } else {
        pk.up(cg.data(), cg.size(), &d_cg);
        pk.up(quad->xref, (size_t)2 * nq, &d_xq);
        pk.up(quad->w, (size_t)nq, &d_wq);
    }
    SG_TRY(pk.commit(ctx, ctx->w_samp));
    // Psi at the full sample y[1:M]: the context's rows are [S][M1] with y_{s,0} = 1 first
    SG_TRY(launch_psi(ctx, &sorted, d_mi, d_rec, d_norms, ctx->d_y64, ctx->M1, 1, (int)M, (int)S, d_psi, lds));
    if (qf) {
        QfArgs b{};
        b.ncells = (int)nc;
        b.S = (int)S;
        b.ld = (int)ctx->ld;
        b.M = (int)M;
        b.nsg = (int)nsg;
        b.groups = groups;
        b.lds = lds;
        b.vol = d_vol;
        b.KT = d_KT;
        b.E = d_E;
        b.Mq = d_Mq;
        b.ddofs = d_dd;
        b.sdofs = d_sd;
        b.D = (const double*)ctx->w_vec[10].p;
        b.U = d_U;
        b.psi = d_psi;
        b.kptr = d_kptr;
        b.part = d_part;
        int rc;
        if (ndd == 6 && nds == 3) rc = launch_error_qf<6, 3>(ctx, b, blocks, smem_qf);
        else if (ndd == 6) rc = launch_error_qf<6, 6>(ctx, b, blocks, smem_qf);
        else rc = launch_error_qf<3, 3>(ctx, b, blocks, smem_qf);
        SG_TRY(rc);
        ctx->sampling_form = 1;
    } else {
        ctx->sampling_form = 2;
        ErrArgs a{};
        a.od = mesh->order;
        a.os = sg_space->order;
        a.nq = nq;
        a.ncells = (int)nc;
        a.S = (int)S;
        a.ld = (int)ctx->ld;
        a.M = (int)M;
        a.nsg = (int)nsg;
        a.groups = groups;
        a.lds = lds;
        a.cg = d_cg;
        a.ddofs = d_dd;
        a.sdofs = d_sd;
        a.D = (const double*)ctx->w_vec[10].p;
        a.U = d_U;
        a.psi = d_psi;
        a.kptr = d_kptr;
        a.xq = d_xq;
        a.wq = d_wq;
        a.part = d_part;
        int rc;
        if (ndd == 6 && nds == 3) rc = launch_error<6, 3>(ctx, a, blocks, smem);
        else if (ndd == 6) rc = launch_error<6, 6>(ctx, a, blocks, smem);
        else if (nds == 3) rc = launch_error<3, 3>(ctx, a, blocks, smem);
        else rc = launch_error<3, 6>(ctx, a, blocks, smem);
        SG_TRY(rc);
    }
    k_sampling_reduce<<<(int)((per + 255) / 256), 256, 0, ctx->stream>>>(d_part, groups, (int)M, (int)S, d_eh, d_el);
    SG_LAUNCHED(ctx);
    SG_CUDA(ctx, cudaMemcpyAsync(errH1, d_eh, (size_t)(M + 1) * S * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    SG_CUDA(ctx, cudaMemcpyAsync(errL2, d_el, (size_t)(M + 1) * S * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    SG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return SGFEM_OK;
}

extern "C" const char* sgfem_sampling_error_log(const sgfem_context* ctx) {
    if (!ctx) return "no context";
    return ctx->sampling_form == 1 ? "quadratic forms" : ctx->sampling_form == 2 ? "quadrature points" : "none";
}
