// K4: residual error estimator for PoissonProblemPrimal on sm_103a.
//
// estimate(::Type{PoissonProblemPrimal}, sol, C; rhs, bonus_quadorder,
// tail_extension), src/estimate.jl:260-418:
//   volume term (estimate.jl:308-366), per cell T and extended mode j
//       eta_T,j = |T|^3 (active j) or |T| (inactive j) * sum_q w_q ft(x_q)^2
//       ft = [j == 0] f + sum_{(m, nu, g) in list_j} a_m g Laplace(u_nu)   (order > 1)
//   jump term (estimate.jl:370-415), per interior face F
//       J_F,j = |F| * int_F |sum_{(m, nu, g) in list_j} a_m g [[grad u_nu]]|^2
//               (times |F| for active j, divided by |F| for inactive j)
//       added to both neighbouring cells and to eta4modes.
// list_j holds the couplings of extended mode j to ACTIVE modes: the K_0 term
// (0, j, 1) when j is active and (m, nu, G_ext) for active neighbours j +/- e_m.
// Mapping: one warp per cell (volume) or per face (jumps).  Per cell the warp
// first computes Laplace(u_nu) for all active modes and a_m at the quadrature
// points into shared memory, then lanes run over a chunk of extended modes;
// per face it computes the gradient jumps of all active modes at the face
// quadrature points once, then lanes run over the chunk of extended modes.
// Face values go to a chunk buffer and each cell gathers its three faces in a
// fixed order; per-mode sums use fixed-order block reductions (no atomics, so
// results are bitwise reproducible).  FP64 throughout.
#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

#include "fe_basis.cuh"
#include "sgfem_internal.h"

namespace {

constexpr int EW = 4;  // warps per block

struct CellGeo {   // per cell: x0, J (columns p1-p0, p2-p0), grad lambda_0..2, volume
    double x0, y0, j00, j10, j01, j11, g[6], vol;
};

struct FaceGeo {
    int c0, c1;            // neighbouring cells (c1 = -1: boundary face)
    int a0, b0, a1, b1;    // local vertex index of the face nodes A, B in c0 and c1
    double ax, ay, bx, by; // A and B
    double vol;
};

struct Coef {
    int M;                 // terms 0..M
    double freq_pi;
    const double* d;       // d[m], m = 0..M (d[0] unused)
    const int* b1;
    const int* b2;
    double mean;
};

__device__ __forceinline__ double am(const Coef& c, int m, double x, double y) {
    if (m == 0) return c.mean;
    return c.d[m] * cos(c.freq_pi * c.b1[m] * x) * cos(c.freq_pi * c.b2[m] * y);
}

// Laplacians (P2; zero for P1) of the local basis from grad lambda
__device__ __forceinline__ void p2_laplacians(const double* g, double* lap) {
    const int ea[3] = {0, 1, 2}, eb[3] = {1, 2, 0};
    for (int i = 0; i < 3; ++i) lap[i] = 4.0 * (g[2 * i] * g[2 * i] + g[2 * i + 1] * g[2 * i + 1]);
    for (int e = 0; e < 3; ++e)
        lap[3 + e] = 8.0 * (g[2 * ea[e]] * g[2 * eb[e]] + g[2 * ea[e] + 1] * g[2 * eb[e] + 1]);
}

using sgfem_fe::basis_grad;

struct EstArgs {
    int order, nd, nq, nqf, P, Pext, ncells, nfaces, ld;
    const CellGeo* cg;
    const int* cdofs;      // nd per cell, device rows
    const int* cfaces;     // 3 per cell
    const FaceGeo* fg;
    const double* xq;      // 2 x nq reference points
    const double* wq;
    const double* tf;
    const double* wf;
    const double* fqp;     // nq x ncells
    const int* lptr;       // P_ext + 1
    const int* lm;
    const int* lnu;        // device column of the active mode
    const double* lg;
    const double* U;       // device layout, FP64
    Coef coef;
};

// volume term for modes [j0, j1): eta4cell[c + j ncells]
__global__ void __launch_bounds__(EW * 32) k_est_volume(EstArgs a, int j0, int j1, double* __restrict__ eta4cell) {
    extern __shared__ double esm[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int per = a.P + (a.coef.M + 1) * a.nq;
    double* dU = esm + (size_t)warp * per;
    double* A = dU + a.P;
    for (int c = blockIdx.x * EW + warp; c < a.ncells; c += gridDim.x * EW) {
        const CellGeo G = a.cg[c];
        const double v = G.vol;
        if (a.order > 1) {
            double lap[6];
            p2_laplacians(G.g, lap);
            const int* dofs = a.cdofs + (size_t)c * a.nd;
            for (int nu = lane; nu < a.P; nu += 32) {
                double s = 0.0;
                for (int d = 0; d < a.nd; ++d) s = fma(a.U[(size_t)dofs[d] * a.ld + nu], lap[d], s);
                dU[nu] = s;
            }
            for (int t = lane; t < (a.coef.M + 1) * a.nq; t += 32) {
                const int m = t / a.nq, q = t - m * a.nq;
                const double xi = a.xq[2 * q], eta = a.xq[2 * q + 1];
                const double x = G.x0 + G.j00 * xi + G.j01 * eta, y = G.y0 + G.j10 * xi + G.j11 * eta;
                A[t] = am(a.coef, m, x, y);
            }
        }
        __syncwarp();
        for (int j = j0 + lane; j < j1; j += 32) {
            double acc = 0.0;
            for (int q = 0; q < a.nq; ++q) {
                double ft = (j == 0) ? a.fqp[(size_t)c * a.nq + q] : 0.0;
                if (a.order > 1)
                    for (int e = a.lptr[j]; e < a.lptr[j + 1]; ++e)
                        ft = fma(A[a.lm[e] * a.nq + q] * a.lg[e], dU[a.lnu[e]], ft);
                acc = fma(a.wq[q] * ft, ft, acc);
            }
            eta4cell[(size_t)j * a.ncells + c] = acc * (j < a.P ? v * v * v : v);
        }
        __syncwarp();
    }
}

// jump term for modes [j0, j1): jumps[(j - j0) nfaces + f]
__global__ void __launch_bounds__(EW * 32) k_est_faces(EstArgs a, int j0, int j1, double* __restrict__ jumps) {
    extern __shared__ double esm[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int per = 2 * a.P * a.nqf + (a.coef.M + 1) * a.nqf + 2 * a.nqf * 12;
    double* J = esm + (size_t)warp * per;       // [nu][q][2]
    double* A = J + 2 * a.P * a.nqf;            // [m][q]
    double* BG = A + (a.coef.M + 1) * a.nqf;    // [side][q][12]
    for (int f = blockIdx.x * EW + warp; f < a.nfaces; f += gridDim.x * EW) {
        const FaceGeo F = a.fg[f];
        if (F.c1 < 0) {
            for (int j = j0 + lane; j < j1; j += 32) jumps[(size_t)(j - j0) * a.nfaces + f] = 0.0;
            continue;
        }
        for (int t = lane; t < (a.coef.M + 1) * a.nqf; t += 32) {
            const int m = t / a.nqf, q = t - m * a.nqf;
            const double s = a.tf[q];
            A[t] = am(a.coef, m, (1.0 - s) * F.ax + s * F.bx, (1.0 - s) * F.ay + s * F.by);
        }
        for (int t = lane; t < 2 * a.nqf; t += 32) {
            const int side = t / a.nqf, q = t - side * a.nqf;
            const CellGeo G = a.cg[side ? F.c1 : F.c0];
            double lam[3] = {0.0, 0.0, 0.0};
            const double s = a.tf[q];
            lam[side ? F.a1 : F.a0] = 1.0 - s;
            lam[side ? F.b1 : F.b0] = s;
            basis_grad(a.order, G.g, lam, BG + (size_t)t * 12);
        }
        __syncwarp();
        const int* d0 = a.cdofs + (size_t)F.c0 * a.nd;
        const int* d1 = a.cdofs + (size_t)F.c1 * a.nd;
        for (int nu = lane; nu < a.P; nu += 32) {
            double u0[6], u1[6];
            for (int d = 0; d < a.nd; ++d) {
                u0[d] = a.U[(size_t)d0[d] * a.ld + nu];
                u1[d] = a.U[(size_t)d1[d] * a.ld + nu];
            }
            for (int q = 0; q < a.nqf; ++q) {
                const double* b0 = BG + (size_t)q * 12;
                const double* b1 = BG + (size_t)(a.nqf + q) * 12;
                double gx = 0.0, gy = 0.0;
                for (int d = 0; d < a.nd; ++d) {
                    gx = fma(u0[d], b0[2 * d], gx);
                    gy = fma(u0[d], b0[2 * d + 1], gy);
                    gx = fma(-u1[d], b1[2 * d], gx);
                    gy = fma(-u1[d], b1[2 * d + 1], gy);
                }
                J[((size_t)nu * a.nqf + q) * 2] = gx;
                J[((size_t)nu * a.nqf + q) * 2 + 1] = gy;
            }
        }
        __syncwarp();
        for (int j = j0 + lane; j < j1; j += 32) {
            double acc = 0.0;
            for (int q = 0; q < a.nqf; ++q) {
                double vx = 0.0, vy = 0.0;
                for (int e = a.lptr[j]; e < a.lptr[j + 1]; ++e) {
                    const double s = A[a.lm[e] * a.nqf + q] * a.lg[e];
                    const double* jn = J + ((size_t)a.lnu[e] * a.nqf + q) * 2;
                    vx = fma(s, jn[0], vx);
                    vy = fma(s, jn[1], vy);
                }
                acc = fma(a.wf[q], vx * vx + vy * vy, acc);
            }
            const double val = F.vol * acc * (j < a.P ? F.vol : 1.0 / F.vol);
            jumps[(size_t)(j - j0) * a.nfaces + f] = val;
        }
        __syncwarp();
    }
}

__global__ void k_est_gather(const int* __restrict__ cfaces, const double* __restrict__ jumps, int ncells,
                             int nfaces, int j0, int j1, double* __restrict__ eta4cell) {
    const size_t total = (size_t)(j1 - j0) * ncells;
    for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (size_t)gridDim.x * blockDim.x) {
        const int jl = (int)(t / ncells), c = (int)(t - (size_t)jl * ncells);
        const double* jr = jumps + (size_t)jl * nfaces;
        const int* cf = cfaces + (size_t)c * 3;
        eta4cell[(size_t)(j0 + jl) * ncells + c] += jr[cf[0]] + jr[cf[1]] + jr[cf[2]];
    }
}

// out[j] = sum_i src[j * stride + i], i < len, one block per j, fixed order
__global__ void k_colsum(const double* __restrict__ src, size_t stride, int len, double* __restrict__ out) {
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

// extended modes per pass: the per-face gradient jumps and the a_m at the
// quadrature points are computed once per pass, so one pass covers every mode
// unless the face buffer (nfaces x chunk doubles) would exceed ~2 GB
int est_chunk(int64_t nfaces, int64_t Pext) {
    const int64_t cap = std::max<int64_t>(64, ((int64_t)2 << 30) / (8 * std::max<int64_t>(nfaces, 1)));
    return (int)std::max<int64_t>(1, std::min(Pext, cap));
}

template <typename T>
int up(sgfem_context* ctx, std::vector<void*>& owned, const T* src, size_t n, T** dst) {
    void* p = nullptr;
    SG_CUDA(ctx, cudaMalloc(&p, std::max<size_t>(n, 1) * sizeof(T)));
    owned.push_back(p);
    if (n) SG_CUDA(ctx, cudaMemcpyAsync(p, src, n * sizeof(T), cudaMemcpyHostToDevice, ctx->stream));
    *dst = (T*)p;
    return SGFEM_OK;
}

struct Owned {
    std::vector<void*> p;
    ~Owned() {
        for (void* q : p) cudaFree(q);
    }
};

}  // namespace

// host geometry, topology, coefficient terms 0..Mcoef and coupling lists -> device (EstArgs)
static int build_est(sgfem_context* ctx, const double* sol, const sgfem_mesh* mesh, const sgfem_quadrature* quad,
                     const double* f_qp, const sgfem_cosine* coef, const sgfem_extension* ext, int64_t Mcoef,
                     Owned& own, EstArgs& a, std::vector<int>& cfaces_out) {
    SG_TRY(sg_check_ready(ctx));
    if (!sol || !mesh || !quad || !f_qp || !coef || !ext)
        return sg_fail(ctx, SGFEM_ERR_ARGUMENT, "estimator: null argument");
    if (mesh->order != 1 && mesh->order != 2) return sg_fail(ctx, SGFEM_ERR_ARGUMENT, "order must be 1 or 2");
    const int nd = mesh->order == 1 ? 3 : 6;
    const int64_t nc = mesh->ncells, nf = mesh->nfaces, nn = mesh->nnodes;
    if (nc <= 0 || nf <= 0 || nn <= 0 || quad->nq <= 0 || quad->nqf <= 0)
        return sg_fail(ctx, SGFEM_ERR_ARGUMENT, "empty mesh or quadrature");
    const int64_t Pext = ext->P_ext, Mext = ext->M_ext;
    if (Pext < ctx->P || Mext < 0) return sg_fail(ctx, SGFEM_ERR_ARGUMENT, "P_ext < P or M_ext < 0");
    if (Mext > coef->maxm)
        return sg_fail(ctx, SGFEM_ERR_ARGUMENT, "coefficient has fewer terms than the extended multi-indices (maxm < M_ext)");
    SG_CUDA(ctx, cudaSetDevice(ctx->device));

    // ---- host-side geometry and topology (0-based, device rows)
    std::vector<CellGeo> cg(nc);
    std::vector<int> cdofs((size_t)nc * nd), cfaces((size_t)nc * 3);
    for (int64_t c = 0; c < nc; ++c) {
        const int64_t* cn = mesh->cell_nodes + 3 * c;
        double px[3], py[3];
        for (int k = 0; k < 3; ++k) {
            const int64_t v = cn[k] - 1;
            if (v < 0 || v >= nn) return sg_fail(ctx, SGFEM_ERR_ARGUMENT, "cell_nodes out of range");
            px[k] = mesh->coords[2 * v];
            py[k] = mesh->coords[2 * v + 1];
        }
        CellGeo& G = cg[c];
        G.x0 = px[0];
        G.y0 = py[0];
        G.j00 = px[1] - px[0];
        G.j01 = px[2] - px[0];
        G.j10 = py[1] - py[0];
        G.j11 = py[2] - py[0];
        const double det = G.j00 * G.j11 - G.j01 * G.j10;
        if (det == 0.0) return sg_fail(ctx, SGFEM_ERR_ARGUMENT, "degenerate cell");
        // rows of J^-1 are grad xi and grad eta
        const double i00 = G.j11 / det, i01 = -G.j01 / det, i10 = -G.j10 / det, i11 = G.j00 / det;
        G.g[2] = i00; G.g[3] = i01;
        G.g[4] = i10; G.g[5] = i11;
        G.g[0] = -i00 - i10; G.g[1] = -i01 - i11;
        G.vol = mesh->cell_volumes[c];
        for (int d = 0; d < nd; ++d) {
            const int64_t dof = mesh->cell_dofs[(size_t)nd * c + d] - 1;
            if (dof < 0 || dof >= ctx->n) return sg_fail(ctx, SGFEM_ERR_ARGUMENT, "cell_dofs out of range");
            cdofs[(size_t)c * nd + d] = ctx->iperm[dof];
        }
        for (int k = 0; k < 3; ++k) cfaces[(size_t)c * 3 + k] = (int)(mesh->cell_faces[3 * c + k] - 1);
    }
    std::vector<FaceGeo> fg(nf);
    for (int64_t f = 0; f < nf; ++f) {
        FaceGeo& F = fg[f];
        const int64_t A = mesh->face_nodes[2 * f] - 1, B = mesh->face_nodes[2 * f + 1] - 1;
        F.ax = mesh->coords[2 * A];
        F.ay = mesh->coords[2 * A + 1];
        F.bx = mesh->coords[2 * B];
        F.by = mesh->coords[2 * B + 1];
        F.vol = mesh->face_volumes[f];
        F.c0 = (int)(mesh->face_cells[2 * f] - 1);
        F.c1 = (int)(mesh->face_cells[2 * f + 1] - 1);
        if (F.c0 < 0) std::swap(F.c0, F.c1);
        if (F.c0 < 0) return sg_fail(ctx, SGFEM_ERR_ARGUMENT, "face without a cell");
        int* loc[2][2] = {{&F.a0, &F.b0}, {&F.a1, &F.b1}};
        for (int s = 0; s < 2; ++s) {
            const int c = s ? F.c1 : F.c0;
            *loc[s][0] = *loc[s][1] = 0;
            if (c < 0) continue;
            const int64_t* cn = mesh->cell_nodes + 3 * c;
            int fa = -1, fb = -1;
            for (int k = 0; k < 3; ++k) {
                if (cn[k] - 1 == A) fa = k;
                if (cn[k] - 1 == B) fb = k;
            }
            if (fa < 0 || fb < 0) return sg_fail(ctx, SGFEM_ERR_ARGUMENT, "face nodes not in the neighbouring cell");
            *loc[s][0] = fa;
            *loc[s][1] = fb;
        }
    }
    // coefficient terms 0..Mcoef (>= M_ext)
    if (Mcoef < Mext || Mcoef > coef->maxm) return sg_fail(ctx, SGFEM_ERR_ARGUMENT, "coefficient terms out of range");
    std::vector<double> d(Mcoef + 1, 0.0);
    std::vector<int> b1(Mcoef + 1, 0), b2(Mcoef + 1, 0);
    for (int64_t m = 1; m <= Mcoef; ++m) {
        d[m] = coef->decay_factors[m - 1];
        b1[m] = (int)coef->b1[m - 1];
        b2[m] = (int)coef->b2[m - 1];
    }
    // coupling lists with device columns
    const int64_t L = ext->ptr[Pext];
    std::vector<int> lptr(Pext + 1), lm(L), lnu(L);
    std::vector<double> lg(ext->g, ext->g + L);
    for (int64_t j = 0; j <= Pext; ++j) lptr[j] = (int)ext->ptr[j];
    for (int64_t e = 0; e < L; ++e) {
        if (ext->m[e] < 0 || ext->m[e] > Mext || ext->nu[e] < 0 || ext->nu[e] >= ctx->P)
            return sg_fail(ctx, SGFEM_ERR_ARGUMENT, "extension coupling out of range");
        lm[e] = ext->m[e];
        lnu[e] = ctx->imode[ext->nu[e]];
    }

    // ---- device data
    a = EstArgs{};
    a.order = mesh->order;
    a.nd = nd;
    a.nq = quad->nq;
    a.nqf = quad->nqf;
    a.P = (int)ctx->P;
    a.Pext = (int)Pext;
    a.ncells = (int)nc;
    a.nfaces = (int)nf;
    a.ld = (int)ctx->ld;
    CellGeo* dcg; int* dcd; int* dcf; FaceGeo* dfg; double *dxq, *dwq, *dtf, *dwf, *dfq, *dd, *dlg; int *db1, *db2, *dlp, *dlm, *dln;
    SG_TRY(up(ctx, own.p, cg.data(), cg.size(), &dcg));
    SG_TRY(up(ctx, own.p, cdofs.data(), cdofs.size(), &dcd));
    SG_TRY(up(ctx, own.p, cfaces.data(), cfaces.size(), &dcf));
    SG_TRY(up(ctx, own.p, fg.data(), fg.size(), &dfg));
    SG_TRY(up(ctx, own.p, quad->xref, (size_t)2 * quad->nq, &dxq));
    SG_TRY(up(ctx, own.p, quad->w, (size_t)quad->nq, &dwq));
    SG_TRY(up(ctx, own.p, quad->tref, (size_t)quad->nqf, &dtf));
    SG_TRY(up(ctx, own.p, quad->wf, (size_t)quad->nqf, &dwf));
    SG_TRY(up(ctx, own.p, f_qp, (size_t)quad->nq * nc, &dfq));
    SG_TRY(up(ctx, own.p, d.data(), d.size(), &dd));
    SG_TRY(up(ctx, own.p, b1.data(), b1.size(), &db1));
    SG_TRY(up(ctx, own.p, b2.data(), b2.size(), &db2));
    SG_TRY(up(ctx, own.p, lptr.data(), lptr.size(), &dlp));
    SG_TRY(up(ctx, own.p, lm.data(), lm.size(), &dlm));
    SG_TRY(up(ctx, own.p, lnu.data(), lnu.size(), &dln));
    SG_TRY(up(ctx, own.p, lg.data(), lg.size(), &dlg));
    a.cg = dcg; a.cdofs = dcd; a.cfaces = dcf; a.fg = dfg; a.xq = dxq; a.wq = dwq; a.tf = dtf; a.wf = dwf; a.fqp = dfq;
    a.lptr = dlp; a.lm = dlm; a.lnu = dln; a.lg = dlg;
    a.coef = Coef{(int)Mext, M_PI * coef->freq, dd, db1, db2, coef->mean};
    cfaces_out = cfaces;
    // solution in the device layout
    const size_t vb = sg_vec_bytes(ctx, SGFEM_FP64);
    SG_TRY(sg_ensure(ctx, ctx->w_vec[11], vb));
    SG_TRY(sgfem_to_device_layout(ctx, sol, ctx->w_vec[11].p, SGFEM_FP64));
    a.U = (const double*)ctx->w_vec[11].p;

    return SGFEM_OK;
}

extern "C" int sgfem_estimate_primal(sgfem_context* ctx, const double* sol, const sgfem_mesh* mesh,
                                     const sgfem_quadrature* quad, const double* f_qp, const sgfem_cosine* coef,
                                     const sgfem_extension* ext, double* eta4modes, double* eta4cell) {
    if (!eta4modes || !eta4cell) return sg_fail(ctx, SGFEM_ERR_ARGUMENT, "sgfem_estimate_primal: null argument");
    Owned own;
    EstArgs a{};
    std::vector<int> cfh;
    SG_TRY(build_est(ctx, sol, mesh, quad, f_qp, coef, ext, ext ? ext->M_ext : 0, own, a, cfh));
    const int64_t nc = a.ncells, nf = a.nfaces, Pext = a.Pext, Mext = a.coef.M;
    const int* dcf = a.cfaces;
    const int chunk = est_chunk(nf, Pext);
    double *d_eta, *d_jumps, *d_vsum, *d_jsum;
    SG_CUDA(ctx, cudaMalloc((void**)&d_eta, (size_t)nc * Pext * sizeof(double)));
    own.p.push_back(d_eta);
    SG_CUDA(ctx, cudaMalloc((void**)&d_jumps, (size_t)nf * chunk * sizeof(double)));
    own.p.push_back(d_jumps);
    SG_CUDA(ctx, cudaMalloc((void**)&d_vsum, (size_t)Pext * sizeof(double)));
    own.p.push_back(d_vsum);
    SG_CUDA(ctx, cudaMalloc((void**)&d_jsum, (size_t)Pext * sizeof(double)));
    own.p.push_back(d_jsum);

    const size_t smem_v = (size_t)EW * (a.P + (Mext + 1) * a.nq) * sizeof(double);
    const size_t smem_f = (size_t)EW * (2 * a.P * a.nqf + (Mext + 1) * a.nqf + 2 * a.nqf * 12) * sizeof(double);
    if (smem_v > 220 * 1024 || smem_f > 220 * 1024)
        return sg_fail(ctx, SGFEM_ERR_UNSUPPORTED, "estimator: too many modes or quadrature points for shared memory");
    if (smem_v > 48 * 1024)
        SG_CUDA(ctx, cudaFuncSetAttribute(k_est_volume, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_v));
    if (smem_f > 48 * 1024)
        SG_CUDA(ctx, cudaFuncSetAttribute(k_est_faces, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_f));
    const int gv = (int)std::min<int64_t>((nc + EW - 1) / EW, (int64_t)ctx->num_sms * 16);
    const int gf = (int)std::min<int64_t>((nf + EW - 1) / EW, (int64_t)ctx->num_sms * 16);
    for (int j0 = 0; j0 < Pext; j0 += chunk) {
        const int j1 = (int)std::min<int64_t>(Pext, j0 + chunk);
        k_est_volume<<<gv, EW * 32, smem_v, ctx->stream>>>(a, j0, j1, d_eta);
        SG_LAUNCHED(ctx);
        k_colsum<<<j1 - j0, 256, 0, ctx->stream>>>(d_eta + (size_t)j0 * nc, (size_t)nc, (int)nc, d_vsum + j0);
        SG_LAUNCHED(ctx);
        k_est_faces<<<gf, EW * 32, smem_f, ctx->stream>>>(a, j0, j1, d_jumps);
        SG_LAUNCHED(ctx);
        k_colsum<<<j1 - j0, 256, 0, ctx->stream>>>(d_jumps, (size_t)nf, (int)nf, d_jsum + j0);
        SG_LAUNCHED(ctx);
        const int gg = (int)std::min<int64_t>(((int64_t)(j1 - j0) * nc + 255) / 256, (int64_t)ctx->num_sms * 16);
        k_est_gather<<<gg, 256, 0, ctx->stream>>>(dcf, d_jumps, (int)nc, (int)nf, j0, j1, d_eta);
        SG_LAUNCHED(ctx);
    }
    std::vector<double> vsum(Pext), jsum(Pext);
    SG_CUDA(ctx, cudaMemcpyAsync(vsum.data(), d_vsum, Pext * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    SG_CUDA(ctx, cudaMemcpyAsync(jsum.data(), d_jsum, Pext * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    SG_CUDA(ctx, cudaMemcpyAsync(eta4cell, d_eta, (size_t)nc * Pext * sizeof(double), cudaMemcpyDeviceToHost,
                                 ctx->stream));
    SG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    for (int64_t j = 0; j < Pext; ++j) eta4modes[j] = std::sqrt(vsum[j] + jsum[j]);
    return SGFEM_OK;
}

// ---------------------------------------------------------------------------
// estimate(::Type{LogTransformedPoissonProblemPrimal}, sol, C; rhs,
// bonus_quadorder, tail_extension), src/estimate.jl:70-257.
//   volume term (:178-214), per cell T, extended mode j, quadrature point q:
//       r = lambda_j(x_q) f(x_q) [+ Laplace(u_j) for P2 and active j]
//           + sum_{(m >= 1, nu, g) in list_j} g grad a_m(x_q) . grad u_nu(x_q)
//       eta_T,j = sum_q w_q r^2 times |T|^2 (active j) or |T| (inactive j)
//   lambda_j: the interpolant (degree iorder on the cells) of the Hermite chaos
//   coefficient of exp(-a) (:102-114), given by its values at the interpolation dofs;
//   data term (:139-156): zeta1 = sum_T sum_q f^2 exp(2 sum_{m<=maxm} a_m^2) w |T|,
//   zeta2 = sum_T sum_q sum_j lambda_j^2 f^2 w |T|;
//   jump term (:231-246): for active j, |F| int_F |[[grad u_j]]|^2 on interior faces,
//   added to the adjacent cells; eta4modes[j] = sqrt(V_j) + sqrt(V_j + J_j).
namespace {

struct LogArgs {
    int iorder, ndi, Mext, maxm;
    const int* idofs;       // ndi per cell, 0-based
    const double* lamv;     // [j][ndofs_i]
    long long ndofs_i;
};

__global__ void __launch_bounds__(EW * 32) k_elog_volume(EstArgs a, LogArgs l, int j0, int j1,
                                                          double* __restrict__ eta4cell, double* __restrict__ z1,
                                                          double* __restrict__ z2) {
    extern __shared__ double esm[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int per = 2 * a.P * a.nq + a.P + 2 * l.Mext * a.nq + a.nq * 6 + a.nq;
    double* GU = esm + (size_t)warp * per;     // [nu][q][2] grad u_nu
    double* LU = GU + 2 * a.P * a.nq;          // [nu] Laplace u_nu (P2)
    double* GA = LU + a.P;                     // [m-1][q][2] grad a_m
    double* PI = GA + 2 * l.Mext * a.nq;       // [q][ndi] interpolation basis values
    double* FQ = PI + a.nq * 6;                // [q] f
    for (int c = blockIdx.x * EW + warp; c < a.ncells; c += gridDim.x * EW) {
        const CellGeo G = a.cg[c];
        const double v = G.vol;
        const int* dofs = a.cdofs + (size_t)c * a.nd;
        for (int t = lane; t < a.P * a.nq; t += 32) {
            const int nu = t / a.nq, q = t - nu * a.nq;
            const double lam[3] = {1.0 - a.xq[2 * q] - a.xq[2 * q + 1], a.xq[2 * q], a.xq[2 * q + 1]};
            double gg[12];
            basis_grad(a.order, G.g, lam, gg);
            double gx = 0.0, gy = 0.0;
            for (int d = 0; d < a.nd; ++d) {
                const double u = a.U[(size_t)dofs[d] * a.ld + nu];
                gx = fma(u, gg[2 * d], gx);
                gy = fma(u, gg[2 * d + 1], gy);
            }
            GU[2 * t] = gx;
            GU[2 * t + 1] = gy;
        }
        if (a.order > 1) {
            double lap[6];
            p2_laplacians(G.g, lap);
            for (int nu = lane; nu < a.P; nu += 32) {
                double s = 0.0;
                for (int d = 0; d < a.nd; ++d) s = fma(a.U[(size_t)dofs[d] * a.ld + nu], lap[d], s);
                LU[nu] = s;
            }
        }
        for (int t = lane; t < l.Mext * a.nq; t += 32) {
            const int m = 1 + t / a.nq, q = t % a.nq;
            const double xi = a.xq[2 * q], eta = a.xq[2 * q + 1];
            const double x = G.x0 + G.j00 * xi + G.j01 * eta, y = G.y0 + G.j10 * xi + G.j11 * eta;
            // grad a_m = d_m (-b1 w sin(b1 w x) cos(b2 w y), -b2 w cos(b1 w x) sin(b2 w y)), w = freq pi
            const double w = a.coef.freq_pi, bx = a.coef.b1[m] * w, by = a.coef.b2[m] * w;
            double sx, cx, sy, cy;
            sincos(bx * x, &sx, &cx);
            sincos(by * y, &sy, &cy);
            GA[2 * t] = -a.coef.d[m] * bx * sx * cy;
            GA[2 * t + 1] = -a.coef.d[m] * by * cx * sy;
        }
        for (int q = lane; q < a.nq; q += 32) {
            const double lam[3] = {1.0 - a.xq[2 * q] - a.xq[2 * q + 1], a.xq[2 * q], a.xq[2 * q + 1]};
            double pv[6];
            sgfem_fe::basis_val(l.iorder, lam, pv);
            for (int d = 0; d < l.ndi; ++d) PI[q * 6 + d] = pv[d];
            FQ[q] = a.fqp[(size_t)c * a.nq + q];
        }
        __syncwarp();
        // data term zeta1 (first chunk only): lanes over quadrature points
        if (j0 == 0) {
            double zz = 0.0;
            for (int q = lane; q < a.nq; q += 32) {
                const double xi = a.xq[2 * q], eta = a.xq[2 * q + 1];
                const double x = G.x0 + G.j00 * xi + G.j01 * eta, y = G.y0 + G.j10 * xi + G.j11 * eta;
                double km = 0.0;
                for (int m = 1; m <= l.maxm; ++m) {
                    const double am_ = a.coef.d[m] * cos(a.coef.freq_pi * a.coef.b1[m] * x) *
                                       cos(a.coef.freq_pi * a.coef.b2[m] * y);
                    km = fma(am_, am_, km);
                }
                zz += FQ[q] * FQ[q] * exp(2.0 * km) * a.wq[q] * v;
            }
            for (int o = 16; o > 0; o >>= 1) zz += __shfl_down_sync(0xffffffffu, zz, o);
            if (lane == 0) z1[c] = zz;
        }
        const int* idofs = l.idofs + (size_t)c * l.ndi;
        double zacc = 0.0;
        for (int j = j0 + lane; j < j1; j += 32) {
            const double* lj = l.lamv + (size_t)j * l.ndofs_i;
            double lnode[6];
            for (int d = 0; d < l.ndi; ++d) lnode[d] = lj[idofs[d]];
            double acc = 0.0;
            for (int q = 0; q < a.nq; ++q) {
                double lam = 0.0;
                for (int d = 0; d < l.ndi; ++d) lam = fma(PI[q * 6 + d], lnode[d], lam);
                double r = lam * FQ[q];
                zacc += lam * lam * FQ[q] * FQ[q] * a.wq[q] * v;
                if (a.order > 1 && j < a.P) r += LU[j];
                for (int e = a.lptr[j]; e < a.lptr[j + 1]; ++e) {
                    const int m = a.lm[e];
                    if (m == 0) continue;
                    const double* ga = GA + 2 * ((m - 1) * a.nq + q);
                    const double* gu = GU + 2 * (a.lnu[e] * a.nq + q);
                    r = fma(a.lg[e], ga[0] * gu[0] + ga[1] * gu[1], r);
                }
                acc = fma(a.wq[q] * r, r, acc);
            }
            eta4cell[(size_t)j * a.ncells + c] = acc * (j < a.P ? v * v : v);
        }
        for (int o = 16; o > 0; o >>= 1) zacc += __shfl_down_sync(0xffffffffu, zacc, o);
        if (lane == 0) z2[c] += zacc;
        __syncwarp();
    }
}

}  // namespace

extern "C" int sgfem_estimate_logpoisson(sgfem_context* ctx, const double* sol, const sgfem_mesh* mesh,
                                         const sgfem_quadrature* quad, const double* f_qp, const sgfem_cosine* coef,
                                         const sgfem_extension* ext, const sgfem_interpolant* lam,
                                         double* eta4modes, double* eta4cell, double* zeta) {
    if (!eta4modes || !eta4cell || !zeta || !lam || !lam->values || !lam->cell_dofs)
        return sg_fail(ctx, SGFEM_ERR_ARGUMENT, "sgfem_estimate_logpoisson: null argument");
    if (lam->order != 1 && lam->order != 2) return sg_fail(ctx, SGFEM_ERR_ARGUMENT, "interpolation degree 1 or 2");
    Owned own;
    EstArgs a{};
    std::vector<int> cfh;
    SG_TRY(build_est(ctx, sol, mesh, quad, f_qp, coef, ext, coef ? coef->maxm : 0, own, a, cfh));
    const int64_t nc = a.ncells, nf = a.nfaces, Pext = a.Pext;
    const int ndi = sgfem_fe::ndofs4cell(lam->order);
    std::vector<int> idofs((size_t)nc * ndi);
    for (int64_t c = 0; c < nc; ++c)
        for (int d = 0; d < ndi; ++d) {
            const int64_t v = lam->cell_dofs[(size_t)ndi * c + d] - 1;
            if (v < 0 || v >= lam->ndofs) return sg_fail(ctx, SGFEM_ERR_ARGUMENT, "interpolation cell_dofs out of range");
            idofs[(size_t)c * ndi + d] = (int)v;
        }
    for (int64_t t = 0; t < lam->ndofs * Pext; ++t)
        if (!std::isfinite(lam->values[t])) return sg_fail(ctx, SGFEM_ERR_NONFINITE, "non-finite interpolant value");
    LogArgs l{};
    l.iorder = lam->order;
    l.ndi = ndi;
    l.Mext = a.coef.M;
    l.maxm = coef->maxm;
    l.ndofs_i = lam->ndofs;
    int* did;
    double* dlam;
    SG_TRY(up(ctx, own.p, idofs.data(), idofs.size(), &did));
    SG_TRY(up(ctx, own.p, lam->values, (size_t)(lam->ndofs * Pext), &dlam));
    l.idofs = did;
    l.lamv = dlam;
    // a.coef.M = M_ext (gradients); the tables d, b1, b2 hold all maxm terms (data term)

    const int chunk = est_chunk(nf, Pext);
    double *d_eta, *d_jumps, *d_vsum, *d_jsum, *d_z1, *d_z2;
    SG_CUDA(ctx, cudaMalloc((void**)&d_eta, (size_t)nc * Pext * sizeof(double)));
    own.p.push_back(d_eta);
    SG_CUDA(ctx, cudaMalloc((void**)&d_jumps, (size_t)nf * chunk * sizeof(double)));
    own.p.push_back(d_jumps);
    SG_CUDA(ctx, cudaMalloc((void**)&d_vsum, (size_t)Pext * sizeof(double)));
    own.p.push_back(d_vsum);
    SG_CUDA(ctx, cudaMalloc((void**)&d_jsum, (size_t)Pext * sizeof(double)));
    own.p.push_back(d_jsum);
    SG_CUDA(ctx, cudaMalloc((void**)&d_z1, (size_t)nc * sizeof(double)));
    own.p.push_back(d_z1);
    SG_CUDA(ctx, cudaMalloc((void**)&d_z2, (size_t)nc * sizeof(double)));
    own.p.push_back(d_z2);
    SG_CUDA(ctx, cudaMemsetAsync(d_z2, 0, (size_t)nc * sizeof(double), ctx->stream));
    SG_CUDA(ctx, cudaMemsetAsync(d_jsum, 0, (size_t)Pext * sizeof(double), ctx->stream));

    const size_t smem_v = (size_t)EW * (2 * a.P * a.nq + a.P + 2 * l.Mext * a.nq + a.nq * 6 + a.nq) * sizeof(double);
    if (smem_v > 220 * 1024)
        return sg_fail(ctx, SGFEM_ERR_UNSUPPORTED, "estimator: too many modes or quadrature points for shared memory");
    if (smem_v > 48 * 1024)
        SG_CUDA(ctx, cudaFuncSetAttribute(k_elog_volume, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_v));
    const int gv = (int)std::min<int64_t>((nc + EW - 1) / EW, (int64_t)ctx->num_sms * 16);
    for (int j0 = 0; j0 < Pext; j0 += chunk) {
        const int j1 = (int)std::min<int64_t>(Pext, j0 + chunk);
        k_elog_volume<<<gv, EW * 32, smem_v, ctx->stream>>>(a, l, j0, j1, d_eta, d_z1, d_z2);
        SG_LAUNCHED(ctx);
        k_colsum<<<j1 - j0, 256, 0, ctx->stream>>>(d_eta + (size_t)j0 * nc, (size_t)nc, (int)nc, d_vsum + j0);
        SG_LAUNCHED(ctx);
    }
    // jumps of the active modes: unit couplings (0, j, 1), a_0 = 1
    const int P = a.P;
    std::vector<int> jp(Pext + 1, 0), jm(P, 0), jn(P);
    std::vector<double> jg(P, 1.0);
    for (int j = 0; j < P; ++j) {
        jp[j + 1] = j + 1;
        jn[j] = ctx->imode[j];
    }
    for (int64_t j = P; j < Pext; ++j) jp[j + 1] = P;
    int *djp, *djm, *djn;
    double* djg;
    SG_TRY(up(ctx, own.p, jp.data(), jp.size(), &djp));
    SG_TRY(up(ctx, own.p, jm.data(), jm.size(), &djm));
    SG_TRY(up(ctx, own.p, jn.data(), jn.size(), &djn));
    SG_TRY(up(ctx, own.p, jg.data(), jg.size(), &djg));
    EstArgs aj = a;
    aj.lptr = djp;
    aj.lm = djm;
    aj.lnu = djn;
    aj.lg = djg;
    aj.coef.M = 0;
    aj.coef.mean = 1.0;
    const size_t smem_f = (size_t)EW * (2 * aj.P * aj.nqf + aj.nqf + 2 * aj.nqf * 12) * sizeof(double);
    if (smem_f > 220 * 1024) return sg_fail(ctx, SGFEM_ERR_UNSUPPORTED, "estimator: too many modes for the jump term");
    if (smem_f > 48 * 1024)
        SG_CUDA(ctx, cudaFuncSetAttribute(k_est_faces, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_f));
    const int gf = (int)std::min<int64_t>((nf + EW - 1) / EW, (int64_t)ctx->num_sms * 16);
    for (int j0 = 0; j0 < P; j0 += chunk) {
        const int j1 = std::min(P, j0 + chunk);
        k_est_faces<<<gf, EW * 32, smem_f, ctx->stream>>>(aj, j0, j1, d_jumps);
        SG_LAUNCHED(ctx);
        k_colsum<<<j1 - j0, 256, 0, ctx->stream>>>(d_jumps, (size_t)nf, (int)nf, d_jsum + j0);
        SG_LAUNCHED(ctx);
        const int gg = (int)std::min<int64_t>(((int64_t)(j1 - j0) * nc + 255) / 256, (int64_t)ctx->num_sms * 16);
        k_est_gather<<<gg, 256, 0, ctx->stream>>>(a.cfaces, d_jumps, (int)nc, (int)nf, j0, j1, d_eta);
        SG_LAUNCHED(ctx);
    }
    std::vector<double> vsum(Pext), jsum(Pext), z1(nc), z2(nc);
    SG_CUDA(ctx, cudaMemcpyAsync(vsum.data(), d_vsum, Pext * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    SG_CUDA(ctx, cudaMemcpyAsync(jsum.data(), d_jsum, Pext * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    SG_CUDA(ctx, cudaMemcpyAsync(z1.data(), d_z1, nc * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    SG_CUDA(ctx, cudaMemcpyAsync(z2.data(), d_z2, nc * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    SG_CUDA(ctx, cudaMemcpyAsync(eta4cell, d_eta, (size_t)nc * Pext * sizeof(double), cudaMemcpyDeviceToHost,
                                 ctx->stream));
    SG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    for (int64_t j = 0; j < Pext; ++j) {
        eta4modes[j] = std::sqrt(vsum[j]);
        if (j < P) eta4modes[j] += std::sqrt(eta4modes[j] * eta4modes[j] + jsum[j]);
    }
    double s1 = 0.0, s2 = 0.0;
    for (int64_t c = 0; c < nc; ++c) {
        s1 += z1[c];
        s2 += z2[c];
    }
    zeta[0] = s1;
    zeta[1] = s2;
    return SGFEM_OK;
}
