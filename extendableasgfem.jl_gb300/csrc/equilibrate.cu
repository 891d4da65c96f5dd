// Equilibration error estimator of PoissonProblemPrimal on the GPU.
//
// estimate_equilibration(::Type{PoissonProblemPrimal}, sol, C; rhs,
// tail_extension), src/estimate.jl:607-954.  For every node z and every
// extended mode j a local flux sigma_{z,j} of the Raviart-Thomas space RT_k
// (k the order of the H1Pk space: HDIVRTk{2, k}) on the node patch omega_z
// minimises (estimate.jl:760-786)
//     ||sigma - phi_z F_j||^2
//       + sum_T pen sqrt|T| ||div sigma - (F_j . grad phi_z - f phi_z [j = 1])||^2_T,
//     F_j = (a grad u_h)_j = sum_{(m, nu, g) in list_j} g a_m grad u_nu
// (the extended-mode couplings of sgfem_estimate_primal, estimate.jl:733-750),
// over the RT functions on omega_z whose normal flux vanishes on every edge
// that omega_z shares with a cell outside it (the reference pins all dofs of
// the outside cells with a 1e60 diagonal, :792-798, and adds the div-div term
// with the penalty pen = 1e5 instead of a Lagrange multiplier).  The estimate
// (:861-946) per cell and mode is
//     eta_{T,j}^2 = sum_q w_q |T| (|F_j - sigma_j|^2 + (f [j = 1] + div sigma_j)^2 / pi^2),
// sigma_j = sum_z sigma_{z,j}, and eta4modes_j = sqrt(sum_T eta_{T,j}^2).
// Every node patch is its own local problem here; the reference assembles the
// patches of one NodePatchGroups group into one system, which is the same
// problem as long as no two patches of a group share an edge.
//
// RT_k basis of the reference cell (v0 = (0,0), v1 = (1,0), v2 = (0,1)):
// dual to the edge moments int_0^1 sigma(x(t)) . R x'(t) L_l(2t - 1) dt on the
// edges (v0,v1), (v1,v2), (v2,v0) (x(t) from the first vertex to the second, R
// the rotation by -90 degrees, L_l Legendre, l = 0..k) and the interior moments
// int sigma_c q, q in {1} (k = 1) or {1, x, y} (k = 2); built on the host by
// inverting the moment matrix of the monomials of P_k^2 + x P~_k.  The
// contravariant Piola map (J sigma / det J, div / det J) keeps each edge moment
// (J^T R J = det J R), so an edge's moments agree in both cells once they are
// taken along the edge's global direction (lower node to higher node): a cell
// whose local edge runs the other way uses sign (-1)^(l+1).
//
// Device, per chunk of modes: (1) a warp per cell evaluates F_j at its
// quadrature points (lanes over modes); (2) once, a block per patch assembles
// the patch matrix (mass + div-div, the same for all modes) in shared memory
// and factors it (Cholesky); (3) blocks per patch solve the modes of the
// chunk, a thread per mode (the right-hand side is linear in F_j: per-slot
// coefficient tables in shared memory; then two triangular solves), because
// on GB300 every FP64 warp instruction costs the FP64 pipe 16 cycles and a
// warp per mode left most lanes idle; (4) a warp
// per cell adds sigma from its three vertex patches and integrates the
// estimate (lanes over modes).  Fixed summation orders, no atomics: results are
// bitwise reproducible.  FP64 throughout.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "fe_basis.cuh"
#include "sgfem_internal.h"

namespace {

constexpr int QW = 4;        // warps per block of the per-cell kernels
constexpr int QMAX = 16;     // largest cell rule
constexpr int NBMAX = 15;    // RT_2 dofs per cell
constexpr int PMAX = 120;    // largest patch system

struct QCell {
    double x0, y0, j00, j10, j01, j11, g[6], vol, det;
};

struct EqCoef {
    int M;
    double freq_pi, mean;
    const double* d;         // d[m], m = 0..M (d[0] unused)
    const int* b1;
    const int* b2;
};

struct EqArgs {
    int order, nd, nb, nq, ncells, ld;
    const QCell* cg;
    const int* cnode;        // 3 per cell, 0-based
    const int* cdofs;        // nd per cell, device rows
    const signed char* csign;// nb per cell
    const double* xq;        // 2 x nq reference points
    const double* wq;
    const double* fqp;       // nq x ncells
    const double* rtv;       // nq x nb x 2: reference basis values
    const double* rtd;       // nq x nb: reference divergences
    const int* lptr;         // P_ext + 1
    const int* lm;
    const int* lnu;          // device column
    const double* lg;
    const double* U;         // device layout, FP64
    EqCoef coef;
    const int* pptr;         // nnodes + 1: slots of each patch
    const int* pcell;        // slot -> cell
    const unsigned char* ploc; // slot -> local vertex of z in the cell
    const short* pmap;       // slot x nb -> patch dof, -1 = pinned
    const int* pn;           // patch dofs
    const long long* lofs;   // factor offset (n^2 doubles)
    const long long* sofs;   // first dof of the patch in the solution block
    const int* cslot;        // 3 per cell: slot of the cell in the patch of its k-th vertex
    double pen;
    double* FL;              // ncells x nq x nj x 2: F_j at the quadrature points
    double* L;               // Cholesky factors
    double* S;               // (sum of patch dofs) x nj: patch solutions
    int* status;             // bit 0: a patch matrix is not positive definite
};

__device__ __forceinline__ double eq_am(const EqCoef& c, int m, double x, double y) {
    if (m == 0) return c.mean;
    return c.d[m] * cos(c.freq_pi * c.b1[m] * x) * cos(c.freq_pi * c.b2[m] * y);
}

// physical RT basis (Piola, global edge signs) of cell c at every quadrature point:
// bv[(q nb + i) 2 + comp], bd[q nb + i]
__device__ void eq_cell_basis(const EqArgs& a, int c, const QCell& G, double* bv, double* bd, int t0, int dt) {
    const double inv = 1.0 / G.det;
    for (int t = t0; t < a.nq * a.nb; t += dt) {
        const int i = t % a.nb;
        const double s = a.csign[(size_t)c * a.nb + i] * inv;
        const double r0 = a.rtv[2 * t], r1 = a.rtv[2 * t + 1];
        bv[2 * t] = s * (G.j00 * r0 + G.j01 * r1);
        bv[2 * t + 1] = s * (G.j10 * r0 + G.j11 * r1);
        bd[t] = s * a.rtd[t];
    }
}

// (1) F_j at the quadrature points of every cell, modes j0 .. j0 + nj - 1
__global__ void __launch_bounds__(QW * 32) k_eq_flux(EqArgs a, int j0, int nj) {
    extern __shared__ double qsm[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int per = (a.coef.M + 1) * a.nq + a.nq * a.nd * 2;
    double* at = qsm + (size_t)warp * per;
    double* gr = at + (a.coef.M + 1) * a.nq;
    for (int c = blockIdx.x * QW + warp; c < a.ncells; c += gridDim.x * QW) {
        const QCell G = a.cg[c];
        for (int t = lane; t < (a.coef.M + 1) * a.nq; t += 32) {
            const int m = t / a.nq, q = t - m * a.nq;
            const double xi = a.xq[2 * q], eta = a.xq[2 * q + 1];
            at[t] = eq_am(a.coef, m, G.x0 + G.j00 * xi + G.j01 * eta, G.y0 + G.j10 * xi + G.j11 * eta);
        }
        for (int q = lane; q < a.nq; q += 32) {
            const double lam[3] = {1.0 - a.xq[2 * q] - a.xq[2 * q + 1], a.xq[2 * q], a.xq[2 * q + 1]};
            double g12[12];
            sgfem_fe::basis_grad(a.order, G.g, lam, g12);
            for (int k = 0; k < 2 * a.nd; ++k) gr[q * 2 * a.nd + k] = g12[k];
        }
        __syncwarp();
        const int* dofs = a.cdofs + (size_t)c * a.nd;
        for (int jj = lane; jj < nj; jj += 32) {
            const int j = j0 + jj;
            double fx[QMAX], fy[QMAX];
#pragma unroll
            for (int q = 0; q < QMAX; ++q) fx[q] = fy[q] = 0.0;
            for (int e = a.lptr[j]; e < a.lptr[j + 1]; ++e) {
                const int m = a.lm[e];
                const double g = a.lg[e];
                const double* Uc = a.U + a.lnu[e];
                double u[6];
                for (int d = 0; d < a.nd; ++d) u[d] = Uc[(size_t)dofs[d] * a.ld];
#pragma unroll
                for (int q = 0; q < QMAX; ++q) {
                    if (q < a.nq) {
                        double gx = 0.0, gy = 0.0;
                        for (int d = 0; d < a.nd; ++d) {
                            gx = fma(u[d], gr[(q * a.nd + d) * 2], gx);
                            gy = fma(u[d], gr[(q * a.nd + d) * 2 + 1], gy);
                        }
                        const double s = g * at[m * a.nq + q];
                        fx[q] = fma(s, gx, fx[q]);
                        fy[q] = fma(s, gy, fy[q]);
                    }
                }
            }
#pragma unroll
            for (int q = 0; q < QMAX; ++q) {
                if (q < a.nq) {
                    double* o = a.FL + (((size_t)c * a.nq + q) * nj + jj) * 2;
                    o[0] = fx[q];
                    o[1] = fy[q];
                }
            }
        }
        __syncwarp();
    }
}

// (2) patch matrix and its Cholesky factor, one block per patch
__global__ void k_eq_factor(EqArgs a) {
    extern __shared__ double fsm[];
    const int z = blockIdx.x;
    const int n = a.pn[z];
    if (n == 0) return;
    double* A = fsm;
    double* bv = A + (size_t)n * n;
    double* bd = bv + (size_t)a.nq * a.nb * 2;
    for (int t = threadIdx.x; t < n * n; t += blockDim.x) A[t] = 0.0;
    for (int s = a.pptr[z]; s < a.pptr[z + 1]; ++s) {
        const int c = a.pcell[s];
        const QCell G = a.cg[c];
        __syncthreads();
        eq_cell_basis(a, c, G, bv, bd, threadIdx.x, blockDim.x);
        __syncthreads();
        const short* map = a.pmap + (size_t)s * a.nb;
        const double sv = sqrt(G.vol);
        for (int t = threadIdx.x; t < a.nb * a.nb; t += blockDim.x) {
            const int i = t / a.nb, j = t - i * a.nb;
            const int pi = map[i], pj = map[j];
            if (pi < 0 || pj < 0) continue;
            double v = 0.0;
            for (int q = 0; q < a.nq; ++q) {
                const double w = a.wq[q] * G.vol;
                const double* vi = bv + (q * a.nb + i) * 2;
                const double* vj = bv + (q * a.nb + j) * 2;
                v += (vi[0] * vj[0] + vi[1] * vj[1]) * w;
                v += a.pen * sv * w * bd[q * a.nb + i] * bd[q * a.nb + j];
            }
            A[pi * n + pj] += v;
        }
    }
    __syncthreads();
    for (int k = 0; k < n; ++k) {
        if (threadIdx.x == 0) {
            double d = A[k * n + k];
            if (!(d > 0.0)) {
                atomicOr(a.status, 1);
                d = 1.0;
            }
            A[k * n + k] = sqrt(d);
        }
        __syncthreads();
        const double dk = A[k * n + k];
        for (int i = k + 1 + threadIdx.x; i < n; i += blockDim.x) A[i * n + k] /= dk;
        __syncthreads();
        const int r = n - k - 1;
        for (int t = threadIdx.x; t < r * r; t += blockDim.x) {
            const int i = k + 1 + t / r, j = k + 1 + t % r;
            if (j <= i) A[i * n + j] -= A[i * n + k] * A[j * n + k];
        }
        __syncthreads();
    }
    double* Lz = a.L + a.lofs[z];
    for (int t = threadIdx.x; t < n * n; t += blockDim.x) Lz[t] = (t % (n + 1) == 0) ? 1.0 / A[t] : A[t];
}

// (3) the modes of the chunk on one patch, a thread per mode.  The right-hand side
// is linear in F: b_i = sum_{s,q} C[s,q,i] . F_j(s,q) - [j = 0] sum_{s,q} pen_w f phi_z div phi_i
// with C = w phi_z phi_i + pen_w div phi_i grad phi_z (pen_w = pen sqrt|T| w |T|), so
// the block builds C of one slot at a time in shared memory and every thread
// accumulates its own mode's b, then solves L L^T x = b with the factor in
// shared memory (its diagonal stored inverted).  Block (z, g) takes the modes
// g * blockDim.x .. of the chunk.
__global__ void k_eq_solve(EqArgs a, int j0, int nj) {
    extern __shared__ double ssm[];
    const int z = blockIdx.x;
    const int n = a.pn[z];
    if (n == 0) return;
    const int s0 = a.pptr[z], ns = a.pptr[z + 1] - s0;
    const int nt = blockDim.x;
    double* L = ssm;                              // n x n
    double* C = L + (size_t)n * n;                // nq x nb x 2 (one slot)
    double* D = C + (size_t)a.nq * a.nb * 2;      // nb: the f term of one slot
    double* B = D + a.nb;                         // n x nt: b of each thread's mode
    __shared__ int smap[NBMAX];
    const double* Lz = a.L + a.lofs[z];
    for (int t = threadIdx.x; t < n * n; t += nt) L[t] = Lz[t];
    for (int t = threadIdx.x; t < n * nt; t += nt) B[t] = 0.0;
    for (int s = 0; s < ns; ++s) {
        const int c = a.pcell[s0 + s];
        const int loc = a.ploc[s0 + s];
        const QCell G = a.cg[c];
        const double inv = 1.0 / G.det, sv = sqrt(G.vol);
        const short* map = a.pmap + (size_t)(s0 + s) * a.nb;
        __syncthreads();  // the previous slot's tables are no longer read
        for (int i = threadIdx.x; i < a.nb; i += nt) smap[i] = map[i];
        for (int t = threadIdx.x; t < a.nq * a.nb; t += nt) {
            const int q = t / a.nb, i = t - q * a.nb;
            const double sg = a.csign[(size_t)c * a.nb + i] * inv;
            const double r0 = a.rtv[2 * t], r1 = a.rtv[2 * t + 1];
            const double vx = sg * (G.j00 * r0 + G.j01 * r1), vy = sg * (G.j10 * r0 + G.j11 * r1);
            const double dv = sg * a.rtd[t];
            const double xi = a.xq[2 * q], eta = a.xq[2 * q + 1];
            const double phiz = loc == 0 ? 1.0 - xi - eta : (loc == 1 ? xi : eta);
            const double w = a.wq[q] * G.vol;
            const double pw = a.pen * sv * w * dv;
            C[2 * t] = w * phiz * vx + pw * G.g[2 * loc];
            C[2 * t + 1] = w * phiz * vy + pw * G.g[2 * loc + 1];
        }
        if (j0 == 0 && blockIdx.y == 0)  // the f term of mode 0, in quadrature-point order
            for (int i = threadIdx.x; i < a.nb; i += nt) {
                double acc = 0.0;
                for (int q = 0; q < a.nq; ++q) {
                    const int t = q * a.nb + i;
                    const double dv = a.csign[(size_t)c * a.nb + i] * inv * a.rtd[t];
                    const double xi = a.xq[2 * q], eta = a.xq[2 * q + 1];
                    const double phiz = loc == 0 ? 1.0 - xi - eta : (loc == 1 ? xi : eta);
                    const double w = a.wq[q] * G.vol;
                    acc += a.pen * sv * w * dv * a.fqp[(size_t)c * a.nq + q] * phiz;
                }
                D[i] = acc;
            }
        __syncthreads();
        const int jj = blockIdx.y * nt + threadIdx.x;
        if (jj < nj) {
            double* b = B + threadIdx.x;
            const double* fl = a.FL + ((size_t)c * a.nq * nj + jj) * 2;
            for (int q = 0; q < a.nq; ++q) {
                const double fx = fl[(size_t)q * nj * 2], fy = fl[(size_t)q * nj * 2 + 1];
                const double* Cq = C + (size_t)q * a.nb * 2;
                for (int i = 0; i < a.nb; ++i) {
                    const int p = smap[i];
                    if (p >= 0) b[(size_t)p * nt] = fma(Cq[2 * i], fx, fma(Cq[2 * i + 1], fy, b[(size_t)p * nt]));
                }
            }
            if (j0 + jj == 0)
                for (int i = 0; i < a.nb; ++i)
                    if (smap[i] >= 0) b[(size_t)smap[i] * nt] -= D[i];
        }
    }
    __syncthreads();
    double* Sz = a.S + (size_t)a.sofs[z] * nj;
    const int jj = blockIdx.y * nt + threadIdx.x;
    if (jj < nj) {
        double* b = B + threadIdx.x;
        // L y = b, then L^T x = y (diagonal stored inverted)
        for (int i = 0; i < n; ++i) {
            double v = b[(size_t)i * nt];
            for (int k = 0; k < i; ++k) v = fma(-L[i * n + k], b[(size_t)k * nt], v);
            b[(size_t)i * nt] = v * L[i * n + i];
        }
        for (int i = n - 1; i >= 0; --i) {
            double v = b[(size_t)i * nt];
            for (int k = i + 1; k < n; ++k) v = fma(-L[k * n + i], b[(size_t)k * nt], v);
            b[(size_t)i * nt] = v * L[i * n + i];
        }
        for (int p = 0; p < n; ++p) Sz[(size_t)p * nj + jj] = b[(size_t)p * nt];
    }
}

// (4) eta_{T,j}^2 for modes j0 .. j0 + nj - 1: eta4cell[c + j ncells]
__global__ void __launch_bounds__(QW * 32) k_eq_volume(EqArgs a, int j0, int nj, double* __restrict__ eta4cell) {
    extern __shared__ double vsm[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    double* bv = vsm + (size_t)warp * a.nq * a.nb * 3;
    double* bd = bv + (size_t)a.nq * a.nb * 2;
    const double ipi2 = 1.0 / (M_PI * M_PI);
    for (int c = blockIdx.x * QW + warp; c < a.ncells; c += gridDim.x * QW) {
        const QCell G = a.cg[c];
        eq_cell_basis(a, c, G, bv, bd, lane, 32);
        __syncwarp();
        for (int jj = lane; jj < nj; jj += 32) {
            const int j = j0 + jj;
            double cf[NBMAX];
#pragma unroll
            for (int i = 0; i < NBMAX; ++i) cf[i] = 0.0;
            for (int k = 0; k < 3; ++k) {
                const int s = a.cslot[3 * c + k];
                const int z = a.cnode[3 * c + k];
                const short* map = a.pmap + (size_t)s * a.nb;
                const double* Sz = a.S + (size_t)a.sofs[z] * nj + jj;
#pragma unroll
                for (int i = 0; i < NBMAX; ++i) {
                    if (i < a.nb) {
                        const int p = map[i];
                        if (p >= 0) cf[i] += Sz[(size_t)p * nj];
                    }
                }
            }
            double eta = 0.0;
            for (int q = 0; q < a.nq; ++q) {
                double sx = 0.0, sy = 0.0, dv = 0.0;
#pragma unroll
                for (int i = 0; i < NBMAX; ++i) {
                    if (i < a.nb) {
                        sx = fma(cf[i], bv[(q * a.nb + i) * 2], sx);
                        sy = fma(cf[i], bv[(q * a.nb + i) * 2 + 1], sy);
                        dv = fma(cf[i], bd[q * a.nb + i], dv);
                    }
                }
                const double* fl = a.FL + (((size_t)c * a.nq + q) * nj + jj) * 2;
                const double ex = fl[0] - sx, ey = fl[1] - sy;
                const double dd = (j == 0 ? a.fqp[(size_t)c * a.nq + q] : 0.0) + dv;
                eta += (ex * ex + ey * ey + dd * dd * ipi2) * a.wq[q] * G.vol;
            }
            eta4cell[(size_t)j * a.ncells + c] = eta;
        }
        __syncwarp();
    }
}

__global__ void k_eq_colsum(const double* __restrict__ src, size_t stride, int len, double* __restrict__ out) {
    __shared__ double red[256];
    const double* s = src + (size_t)blockIdx.x * stride;
    double v = 0.0;
    for (int i = threadIdx.x; i < len; i += 256) v += s[i];
    red[threadIdx.x] = v;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) out[blockIdx.x] = red[0];
}

// ---- RT_k basis of the reference cell, on the host
struct Poly2 {  // vector polynomial: coefficient of x^a y^b in component c at [c][a][b]
    double v[2][4][4];
};

double mono_int(int a, int b) {  // int_T x^a y^b over the reference triangle
    double num = 1.0, den = 1.0;
    for (int i = 2; i <= a; ++i) num *= i;
    for (int i = 2; i <= b; ++i) num *= i;
    for (int i = 2; i <= a + b + 2; ++i) den *= i;
    return num / den;
}

double poly_eval(const Poly2& p, int c, double x, double y) {
    double s = 0.0, xa = 1.0;
    for (int a = 0; a < 4; ++a, xa *= x) {
        double yb = 1.0;
        for (int b = 0; a + b < 4; ++b, yb *= y) s += p.v[c][a][b] * xa * yb;
    }
    return s;
}

double poly_div(const Poly2& p, double x, double y) {
    double s = 0.0;
    for (int a = 0; a < 4; ++a)
        for (int b = 0; a + b < 4; ++b) {
            if (a > 0) s += a * p.v[0][a][b] * std::pow(x, a - 1) * std::pow(y, b);
            if (b > 0) s += b * p.v[1][a][b] * std::pow(x, a) * std::pow(y, b - 1);
        }
    return s;
}

double legendre01(int l, double t) {
    const double s = 2.0 * t - 1.0;
    return l == 0 ? 1.0 : (l == 1 ? s : 0.5 * (3.0 * s * s - 1.0));
}

// values (nq x nb x 2) and divergences (nq x nb) of the RT_k basis at the points xq
bool rt_basis(int k, int nq, const double* xq, std::vector<double>& val, std::vector<double>& dv) {
    std::vector<Poly2> span;
    for (int c = 0; c < 2; ++c)
        for (int a = 0; a <= k; ++a)
            for (int b = 0; a + b <= k; ++b) {
                Poly2 p{};
                p.v[c][a][b] = 1.0;
                span.push_back(p);
            }
    for (int a = k; a >= 0; --a) {
        Poly2 p{};
        p.v[0][a + 1][k - a] = 1.0;
        p.v[1][a][k - a + 1] = 1.0;
        span.push_back(p);
    }
    const int nb = (int)span.size();
    // moment matrix D[r][j] = N_r(psi_j)
    const double vx[3] = {0.0, 1.0, 0.0}, vy[3] = {0.0, 0.0, 1.0};
    const double gt[4] = {0.0694318442029737124, 0.3300094782075718676, 0.6699905217924281324,
                          0.9305681557970262876};
    const double gw[4] = {0.1739274225687269287, 0.3260725774312730713, 0.3260725774312730713,
                          0.1739274225687269287};
    std::vector<double> D((size_t)nb * nb, 0.0);
    for (int j = 0; j < nb; ++j) {
        int r = 0;
        for (int e = 0; e < 3; ++e) {
            const int va = e, vb = (e + 1) % 3;
            const double dx = vx[vb] - vx[va], dy = vy[vb] - vy[va];
            const double nx = dy, ny = -dx;
            for (int l = 0; l <= k; ++l, ++r) {
                double s = 0.0;
                for (int g = 0; g < 4; ++g) {
                    const double x = vx[va] + gt[g] * dx, y = vy[va] + gt[g] * dy;
                    s += gw[g] * legendre01(l, gt[g]) *
                         (poly_eval(span[j], 0, x, y) * nx + poly_eval(span[j], 1, x, y) * ny);
                }
                D[(size_t)r * nb + j] = s;
            }
        }
        const int qa[3] = {0, 1, 0}, qb[3] = {0, 0, 1};
        const int nqi = k == 1 ? 1 : 3;
        for (int c = 0; c < 2; ++c)
            for (int qi = 0; qi < nqi; ++qi, ++r) {
                double s = 0.0;
                for (int a = 0; a < 4; ++a)
                    for (int b = 0; a + b < 4; ++b)
                        if (span[j].v[c][a][b] != 0.0) s += span[j].v[c][a][b] * mono_int(a + qa[qi], b + qb[qi]);
                D[(size_t)r * nb + j] = s;
            }
    }
    // C = D^-1 (Gauss-Jordan, partial pivoting); basis r = sum_j C[j][r] psi_j
    std::vector<double> C((size_t)nb * nb, 0.0);
    for (int i = 0; i < nb; ++i) C[(size_t)i * nb + i] = 1.0;
    for (int col = 0; col < nb; ++col) {
        int piv = col;
        for (int i = col + 1; i < nb; ++i)
            if (std::fabs(D[(size_t)i * nb + col]) > std::fabs(D[(size_t)piv * nb + col])) piv = i;
        if (std::fabs(D[(size_t)piv * nb + col]) < 1e-14) return false;
        for (int t = 0; t < nb; ++t) {
            std::swap(D[(size_t)col * nb + t], D[(size_t)piv * nb + t]);
            std::swap(C[(size_t)col * nb + t], C[(size_t)piv * nb + t]);
        }
        const double inv = 1.0 / D[(size_t)col * nb + col];
        for (int t = 0; t < nb; ++t) {
            D[(size_t)col * nb + t] *= inv;
            C[(size_t)col * nb + t] *= inv;
        }
        for (int i = 0; i < nb; ++i) {
            if (i == col) continue;
            const double f = D[(size_t)i * nb + col];
            if (f == 0.0) continue;
            for (int t = 0; t < nb; ++t) {
                D[(size_t)i * nb + t] -= f * D[(size_t)col * nb + t];
                C[(size_t)i * nb + t] -= f * C[(size_t)col * nb + t];
            }
        }
    }
    val.assign((size_t)nq * nb * 2, 0.0);
    dv.assign((size_t)nq * nb, 0.0);
    for (int q = 0; q < nq; ++q) {
        const double x = xq[2 * q], y = xq[2 * q + 1];
        std::vector<double> p0(nb), p1(nb), pd(nb);
        for (int j = 0; j < nb; ++j) {
            p0[j] = poly_eval(span[j], 0, x, y);
            p1[j] = poly_eval(span[j], 1, x, y);
            pd[j] = poly_div(span[j], x, y);
        }
        for (int r = 0; r < nb; ++r) {
            double s0 = 0.0, s1 = 0.0, sd = 0.0;
            for (int j = 0; j < nb; ++j) {
                const double cjr = C[(size_t)j * nb + r];
                s0 += cjr * p0[j];
                s1 += cjr * p1[j];
                sd += cjr * pd[j];
            }
            val[((size_t)q * nb + r) * 2] = s0;
            val[((size_t)q * nb + r) * 2 + 1] = s1;
            dv[(size_t)q * nb + r] = sd;
        }
    }
    return true;
}

template <typename T>
int eup(sgfem_context* ctx, std::vector<void*>& owned, const T* src, size_t n, T** dst) {
    void* p = nullptr;
    SG_CUDA(ctx, cudaMalloc(&p, std::max<size_t>(n, 1) * sizeof(T)));
    owned.push_back(p);
    if (n) SG_CUDA(ctx, cudaMemcpyAsync(p, src, n * sizeof(T), cudaMemcpyHostToDevice, ctx->stream));
    *dst = (T*)p;
    return SGFEM_OK;
}

template <typename T>
int ealloc(sgfem_context* ctx, std::vector<void*>& owned, size_t n, T** dst) {
    void* p = nullptr;
    SG_CUDA(ctx, cudaMalloc(&p, std::max<size_t>(n, 1) * sizeof(T)));
    owned.push_back(p);
    *dst = (T*)p;
    return SGFEM_OK;
}

struct EqOwned {
    std::vector<void*> p;
    ~EqOwned() {
        for (void* q : p) cudaFree(q);
    }
};

}  // namespace

extern "C" int sgfem_rt_reference_basis(int k, int np, const double* pts, double* values, double* divs) {
    if ((k != 1 && k != 2) || np < 0 || (np > 0 && (!pts || !values || !divs))) return SGFEM_ERR_ARGUMENT;
    std::vector<double> v, dv;
    if (!rt_basis(k, np, pts, v, dv)) return SGFEM_ERR_UNSUPPORTED;
    std::copy(v.begin(), v.end(), values);
    std::copy(dv.begin(), dv.end(), divs);
    return SGFEM_OK;
}

extern "C" int sgfem_estimate_equilibration(sgfem_context* ctx, const double* sol, const sgfem_mesh* mesh,
                                            const sgfem_quadrature* quad, const double* f_qp,
                                            const sgfem_cosine* coef, const sgfem_extension* ext, double div_penalty,
                                            double* eta4modes, double* eta4cell) {
    SG_TRY(sg_check_ready(ctx));
    char msg[200];
    auto fail = [&](int code, const char* what) {
        snprintf(msg, sizeof(msg), "sgfem_estimate_equilibration: %s", what);
        return sg_fail(ctx, code, msg);
    };
    if (!sol || !mesh || !quad || !f_qp || !coef || !ext || !eta4modes || !eta4cell)
        return fail(SGFEM_ERR_ARGUMENT, "null argument");
    if (mesh->order != 1 && mesh->order != 2) return fail(SGFEM_ERR_ARGUMENT, "order must be 1 or 2");
    if (!(div_penalty > 0.0)) return fail(SGFEM_ERR_ARGUMENT, "div_penalty must be positive");
    const int order = mesh->order, nd = order == 1 ? 3 : 6, nb = order == 1 ? 8 : 15;
    const int64_t nc = mesh->ncells, nn = mesh->nnodes, nf = mesh->nfaces;
    const int nq = quad->nq;
    if (nc <= 0 || nn <= 0 || nf <= 0 || nq <= 0 || nq > QMAX)
        return fail(SGFEM_ERR_ARGUMENT, "empty mesh or cell rule outside 1..16 points");
    const int64_t Pext = ext->P_ext, Mext = ext->M_ext;
    if (Pext < ctx->P || Mext < 0) return fail(SGFEM_ERR_ARGUMENT, "P_ext < P or M_ext < 0");
    if (Mext > coef->maxm) return fail(SGFEM_ERR_ARGUMENT, "coefficient has fewer terms than M_ext");
    SG_CUDA(ctx, cudaSetDevice(ctx->device));

    // ---- cells: geometry, dofs, global edge signs
    std::vector<QCell> cg(nc);
    std::vector<int> cnode((size_t)nc * 3), cdofs((size_t)nc * nd), cface((size_t)nc * 3);
    std::vector<signed char> csign((size_t)nc * nb, 1);
    for (int64_t c = 0; c < nc; ++c) {
        double px[3], py[3];
        for (int k = 0; k < 3; ++k) {
            const int64_t v = mesh->cell_nodes[3 * c + k] - 1;
            if (v < 0 || v >= nn) return fail(SGFEM_ERR_ARGUMENT, "cell_nodes out of range");
            cnode[3 * c + k] = (int)v;
            px[k] = mesh->coords[2 * v];
            py[k] = mesh->coords[2 * v + 1];
        }
        QCell& G = cg[c];
        G.x0 = px[0];
        G.y0 = py[0];
        G.j00 = px[1] - px[0];
        G.j01 = px[2] - px[0];
        G.j10 = py[1] - py[0];
        G.j11 = py[2] - py[0];
        G.det = G.j00 * G.j11 - G.j01 * G.j10;
        if (G.det == 0.0) return fail(SGFEM_ERR_ARGUMENT, "degenerate cell");
        const double i00 = G.j11 / G.det, i01 = -G.j01 / G.det, i10 = -G.j10 / G.det, i11 = G.j00 / G.det;
        G.g[2] = i00; G.g[3] = i01;
        G.g[4] = i10; G.g[5] = i11;
        G.g[0] = -i00 - i10; G.g[1] = -i01 - i11;
        G.vol = mesh->cell_volumes[c];
        for (int d = 0; d < nd; ++d) {
            const int64_t dof = mesh->cell_dofs[(size_t)nd * c + d] - 1;
            if (dof < 0 || dof >= ctx->n) return fail(SGFEM_ERR_ARGUMENT, "cell_dofs out of range");
            cdofs[(size_t)c * nd + d] = ctx->iperm[dof];
        }
        // local edge e runs from local vertex e to e + 1; find its face
        for (int e = 0; e < 3; ++e) {
            const int A = cnode[3 * c + e], B = cnode[3 * c + (e + 1) % 3];
            int face = -1;
            for (int k = 0; k < 3; ++k) {
                const int64_t f = mesh->cell_faces[3 * c + k] - 1;
                if (f < 0 || f >= nf) return fail(SGFEM_ERR_ARGUMENT, "cell_faces out of range");
                const int64_t fa = mesh->face_nodes[2 * f] - 1, fb = mesh->face_nodes[2 * f + 1] - 1;
                if ((fa == A && fb == B) || (fa == B && fb == A)) face = (int)f;
            }
            if (face < 0) return fail(SGFEM_ERR_ARGUMENT, "cell_faces do not match the cell's edges");
            cface[3 * c + e] = face;
            if (A > B)
                for (int l = 0; l <= order; ++l) csign[(size_t)c * nb + e * (order + 1) + l] = (l % 2 == 0) ? -1 : 1;
        }
    }
    // ---- node patches (cells in increasing order) and their dof maps
    std::vector<int> pptr(nn + 1, 0);
    for (int64_t c = 0; c < nc; ++c)
        for (int k = 0; k < 3; ++k) pptr[cnode[3 * c + k] + 1]++;
    for (int64_t z = 0; z < nn; ++z) pptr[z + 1] += pptr[z];
    const int nslots = pptr[nn];
    std::vector<int> pcell(nslots), fillp(pptr.begin(), pptr.end() - 1), cslot((size_t)nc * 3);
    std::vector<unsigned char> ploc(nslots);
    for (int64_t c = 0; c < nc; ++c)
        for (int k = 0; k < 3; ++k) {
            const int z = cnode[3 * c + k];
            const int s = fillp[z]++;
            pcell[s] = (int)c;
            ploc[s] = (unsigned char)k;
            cslot[3 * c + k] = s;
        }
    std::vector<short> pmap((size_t)nslots * nb, -1);
    std::vector<int> pn(nn, 0);
    std::vector<long long> lofs(nn + 1, 0), sofs(nn + 1, 0);
    int n_max = 0;
    for (int64_t z = 0; z < nn; ++z) {
        std::vector<std::pair<int, int>> shared_edges;  // (face * 4 + l, patch dof)
        int cnt = 0;
        for (int s = pptr[z]; s < pptr[z + 1]; ++s) {
            const int c = pcell[s];
            for (int e = 0; e < 3; ++e) {
                const int f = cface[3 * c + e];
                int other = -1;
                for (int t = 0; t < 2; ++t) {
                    const int64_t fc = mesh->face_cells[2 * f + t] - 1;
                    if (fc >= 0 && fc != c) other = (int)fc;
                }
                bool free_edge = other < 0;
                if (!free_edge)
                    for (int k = 0; k < 3; ++k)
                        if (cnode[3 * other + k] == (int)z) free_edge = true;
                if (!free_edge) continue;  // shared with a cell outside the patch: pinned
                for (int l = 0; l <= order; ++l) {
                    const int key = f * 4 + l;
                    int p = -1;
                    for (const auto& se : shared_edges)
                        if (se.first == key) p = se.second;
                    if (p < 0) {
                        p = cnt++;
                        shared_edges.push_back({key, p});
                    }
                    pmap[(size_t)s * nb + e * (order + 1) + l] = (short)p;
                }
            }
            for (int i = 3 * (order + 1); i < nb; ++i) pmap[(size_t)s * nb + i] = (short)(cnt++);
        }
        if (cnt > PMAX) return fail(SGFEM_ERR_UNSUPPORTED, "a node patch has more than 120 flux dofs");
        pn[z] = cnt;
        n_max = std::max(n_max, cnt);
        lofs[z + 1] = lofs[z] + (long long)cnt * cnt;
        sofs[z + 1] = sofs[z] + cnt;
    }
    // ---- RT basis, coefficient, coupling lists
    std::vector<double> rtv, rtd;
    if (!rt_basis(order, nq, quad->xref, rtv, rtd)) return fail(SGFEM_ERR_UNSUPPORTED, "RT moment matrix is singular");
    std::vector<double> d(Mext + 1, 0.0);
    std::vector<int> b1(Mext + 1, 0), b2(Mext + 1, 0);
    for (int64_t m = 1; m <= Mext; ++m) {
        d[m] = coef->decay_factors[m - 1];
        b1[m] = (int)coef->b1[m - 1];
        b2[m] = (int)coef->b2[m - 1];
    }
    const int64_t Lc = ext->ptr[Pext];
    std::vector<int> lptr(Pext + 1), lm(Lc), lnu(Lc);
    std::vector<double> lg(ext->g, ext->g + Lc);
    for (int64_t j = 0; j <= Pext; ++j) lptr[j] = (int)ext->ptr[j];
    for (int64_t e = 0; e < Lc; ++e) {
        if (ext->m[e] < 0 || ext->m[e] > Mext || ext->nu[e] < 0 || ext->nu[e] >= ctx->P)
            return fail(SGFEM_ERR_ARGUMENT, "extension coupling out of range");
        lm[e] = ext->m[e];
        lnu[e] = ctx->imode[ext->nu[e]];
    }
    // ---- launch shapes and the mode chunk (F and the patch solutions of one chunk stay below ~2 GB)
    int dev_smem = 0;
    cudaDeviceGetAttribute(&dev_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, ctx->device);
    const size_t smem_flux = (size_t)QW * ((Mext + 1) * nq + nq * nd * 2) * sizeof(double);
    const size_t smem_fac = ((size_t)n_max * n_max + (size_t)nq * nb * 3) * sizeof(double);
    int st = 128;  // threads (modes) per patch-solve block
    auto sol_bytes = [&](int t) { return ((size_t)n_max * n_max + (size_t)nq * nb * 2 + nb + (size_t)n_max * t) * sizeof(double); };
    while (st > 32 && (int64_t)sol_bytes(st) > dev_smem) st /= 2;
    const size_t smem_sol = sol_bytes(st);
    const size_t smem_vol = (size_t)QW * nq * nb * 3 * sizeof(double);
    if ((int64_t)std::max({smem_flux, smem_fac, smem_sol, smem_vol}) > dev_smem)
        return fail(SGFEM_ERR_UNSUPPORTED, "node patches or coefficient terms too large for shared memory");
    const size_t per_mode = ((size_t)nc * nq * 2 + (size_t)sofs[nn]) * sizeof(double);
    int CH = (int)std::min<int64_t>(Pext, std::max<int64_t>(32, (int64_t)((size_t)2 << 30) / std::max<size_t>(per_mode, 1)));
    if (const char* e = getenv("SGFEM_EQ_CHUNK")) CH = atoi(e);  // modes per pass (tests cover several passes)
    CH = std::max(1, std::min(CH, (int)Pext));

    EqOwned own;
    EqArgs a{};
    a.order = order;
    a.nd = nd;
    a.nb = nb;
    a.nq = nq;
    a.ncells = (int)nc;
    a.ld = (int)ctx->ld;
    a.pen = div_penalty;
    QCell* dcg; int *dcn, *dcd, *dlp, *dlm, *dln, *db1, *db2, *dpp, *dpc, *dpn, *dcs, *dst;
    signed char* dsg; unsigned char* dpl; short* dpm; long long *dlo, *dso;
    double *dxq, *dwq, *dfq, *drv, *drd, *dlg, *dd, *dFL, *dL, *dS, *deta, *dsum;
    SG_TRY(eup(ctx, own.p, cg.data(), cg.size(), &dcg));
    SG_TRY(eup(ctx, own.p, cnode.data(), cnode.size(), &dcn));
    SG_TRY(eup(ctx, own.p, cdofs.data(), cdofs.size(), &dcd));
    SG_TRY(eup(ctx, own.p, csign.data(), csign.size(), &dsg));
    SG_TRY(eup(ctx, own.p, quad->xref, (size_t)2 * nq, &dxq));
    SG_TRY(eup(ctx, own.p, quad->w, (size_t)nq, &dwq));
    SG_TRY(eup(ctx, own.p, f_qp, (size_t)nq * nc, &dfq));
    SG_TRY(eup(ctx, own.p, rtv.data(), rtv.size(), &drv));
    SG_TRY(eup(ctx, own.p, rtd.data(), rtd.size(), &drd));
    SG_TRY(eup(ctx, own.p, lptr.data(), lptr.size(), &dlp));
    SG_TRY(eup(ctx, own.p, lm.data(), lm.size(), &dlm));
    SG_TRY(eup(ctx, own.p, lnu.data(), lnu.size(), &dln));
    SG_TRY(eup(ctx, own.p, lg.data(), lg.size(), &dlg));
    SG_TRY(eup(ctx, own.p, d.data(), d.size(), &dd));
    SG_TRY(eup(ctx, own.p, b1.data(), b1.size(), &db1));
    SG_TRY(eup(ctx, own.p, b2.data(), b2.size(), &db2));
    SG_TRY(eup(ctx, own.p, pptr.data(), pptr.size(), &dpp));
    SG_TRY(eup(ctx, own.p, pcell.data(), pcell.size(), &dpc));
    SG_TRY(eup(ctx, own.p, ploc.data(), ploc.size(), &dpl));
    SG_TRY(eup(ctx, own.p, pmap.data(), pmap.size(), &dpm));
    SG_TRY(eup(ctx, own.p, pn.data(), pn.size(), &dpn));
    SG_TRY(eup(ctx, own.p, lofs.data(), lofs.size(), &dlo));
    SG_TRY(eup(ctx, own.p, sofs.data(), sofs.size(), &dso));
    SG_TRY(eup(ctx, own.p, cslot.data(), cslot.size(), &dcs));
    SG_TRY(ealloc(ctx, own.p, (size_t)nc * nq * CH * 2, &dFL));
    SG_TRY(ealloc(ctx, own.p, (size_t)lofs[nn], &dL));
    SG_TRY(ealloc(ctx, own.p, (size_t)sofs[nn] * CH, &dS));
    SG_TRY(ealloc(ctx, own.p, (size_t)nc * Pext, &deta));
    SG_TRY(ealloc(ctx, own.p, (size_t)Pext, &dsum));
    SG_TRY(ealloc(ctx, own.p, 1, &dst));
    SG_CUDA(ctx, cudaMemsetAsync(dst, 0, sizeof(int), ctx->stream));
    a.cg = dcg; a.cnode = dcn; a.cdofs = dcd; a.csign = dsg; a.xq = dxq; a.wq = dwq; a.fqp = dfq; a.rtv = drv;
    a.rtd = drd; a.lptr = dlp; a.lm = dlm; a.lnu = dln; a.lg = dlg;
    a.coef = EqCoef{(int)Mext, M_PI * coef->freq, coef->mean, dd, db1, db2};
    a.pptr = dpp; a.pcell = dpc; a.ploc = dpl; a.pmap = dpm; a.pn = dpn; a.lofs = dlo; a.sofs = dso; a.cslot = dcs;
    a.FL = dFL; a.L = dL; a.S = dS; a.status = dst;
    // the solution in the device layout
    const size_t vb = sg_vec_bytes(ctx, SGFEM_FP64);
    SG_TRY(sg_ensure(ctx, ctx->w_vec[11], vb));
    SG_TRY(sgfem_to_device_layout(ctx, sol, ctx->w_vec[11].p, SGFEM_FP64));
    a.U = (const double*)ctx->w_vec[11].p;

    if (smem_flux > 48 * 1024)
        SG_CUDA(ctx, cudaFuncSetAttribute(k_eq_flux, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_flux));
    if (smem_fac > 48 * 1024)
        SG_CUDA(ctx, cudaFuncSetAttribute(k_eq_factor, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_fac));
    if (smem_sol > 48 * 1024)
        SG_CUDA(ctx, cudaFuncSetAttribute(k_eq_solve, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_sol));
    if (smem_vol > 48 * 1024)
        SG_CUDA(ctx, cudaFuncSetAttribute(k_eq_volume, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_vol));
    const int gc = (int)std::min<int64_t>((nc + QW - 1) / QW, (int64_t)std::max(ctx->num_sms, 1) * 16);
    k_eq_factor<<<(unsigned)nn, 128, smem_fac, ctx->stream>>>(a);
    SG_LAUNCHED(ctx);
    for (int64_t j0 = 0; j0 < Pext; j0 += CH) {
        const int nj = (int)std::min<int64_t>(CH, Pext - j0);
        k_eq_flux<<<gc, QW * 32, smem_flux, ctx->stream>>>(a, (int)j0, nj);
        SG_LAUNCHED(ctx);
        k_eq_solve<<<dim3((unsigned)nn, (unsigned)((nj + st - 1) / st)), st, smem_sol, ctx->stream>>>(a, (int)j0, nj);
        SG_LAUNCHED(ctx);
        k_eq_volume<<<gc, QW * 32, smem_vol, ctx->stream>>>(a, (int)j0, nj, deta);
        SG_LAUNCHED(ctx);
    }
    k_eq_colsum<<<(unsigned)Pext, 256, 0, ctx->stream>>>(deta, (size_t)nc, (int)nc, dsum);
    SG_LAUNCHED(ctx);
    std::vector<double> sum(Pext);
    int status = 0;
    SG_CUDA(ctx, cudaMemcpyAsync(sum.data(), dsum, Pext * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    SG_CUDA(ctx, cudaMemcpyAsync(eta4cell, deta, (size_t)nc * Pext * sizeof(double), cudaMemcpyDeviceToHost,
                                 ctx->stream));
    SG_CUDA(ctx, cudaMemcpyAsync(&status, dst, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    SG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (status & 1) return fail(SGFEM_ERR_BREAKDOWN, "a node patch matrix is not positive definite");
    for (int64_t j = 0; j < Pext; ++j) eta4modes[j] = std::sqrt(sum[j]);
    return SGFEM_OK;
}
