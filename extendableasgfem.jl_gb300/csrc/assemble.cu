// Stiffness matrices of the affine cosine coefficient, assembled on the GPU
// (and, with the same gather, the convection blocks of the log-transformed
// problem, N_m[i, j] = -(grad a_m . grad phi_j, phi_i), logpoisson_primal.jl:
// 101-107).
//
// K_m = (a_m grad u, grad v), m = m0..m1, on the H1Pk space (P1 / P2) of a
// triangle mesh: the K_m of solve!(PoissonProblemPrimal) (poisson_primal.jl:
// 56-68; the reference assembles them with ExtendableFEM on the host, one
// pass per term) with a_0 = mean and a_m (m >= 1) the cosine terms of
// StochasticCoefficientCosinus (cosinus.jl:11-76).  The sparsity pattern is the
// caller's (the CSC arrays of its SparseMatrixCSC); the values are
//   K_m[i, j] = sum over cells T holding i and j of
//               sum_q w_q |T| a_m(x_q) grad phi_i(x_q) . grad phi_j(x_q)
// with the cell rule (reference points, weights summing to one).
// Host: cell geometry (origin, Jacobian, gradients of the barycentric
// coordinates), and for every nonzero the list of (cell, local row, local
// column) that contribute to it, in increasing cell order (counting sort: the
// integer work).  Device: a_m at the quadrature points of every cell, then one
// thread per nonzero adds its contributions in that order (no atomics, so the
// values are bitwise reproducible and summed in the order of a cell-by-cell
// scatter).  FP64 throughout.
#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <vector>

#include "fe_basis.cuh"
#include "sgfem_internal.h"

namespace {

constexpr int AQ = 16;      // quadrature points per chunk of the gather (one chunk up to 16 points)
constexpr int AQMAX = 1024; // largest cell rule

struct AGeo {
    double x0, y0, j00, j10, j01, j11, g[6], vol;
};

struct AArgs {
    int kind;            // 0: (a_m grad u, grad v); 1: -(grad a_m . grad u, v)
    int order, nd, nq, nc, nterms, m0;
    int64_t nnz;
    const AGeo* geo;
    const double* xq;    // 2 x nq
    const double* wq;
    double freq_pi, mean;
    const double* d;     // d[m - m0] (d of m = 0 unused)
    const int* b1;
    const int* b2;
    double* A;           // nterms x nc x nq: a_m at the quadrature points (kind 1: grad a_m, 2 values)
    const int64_t* eptr; // nnz + 1
    const int* ecell;
    const unsigned char* eab;  // local row * nd + local column
};

__global__ void k_am_qp(AArgs a) {
    const size_t total = (size_t)a.nterms * a.nc * a.nq;
    for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (size_t)gridDim.x * blockDim.x) {
        const int q = (int)(t % a.nq);
        const size_t r = t / a.nq;
        const int c = (int)(r % a.nc);
        const int mi = (int)(r / a.nc);
        const int m = a.m0 + mi;
        double v = a.kind == 0 ? a.mean : 0.0, vy = 0.0;
        if (m > 0) {
            const AGeo& G = a.geo[c];
            const double xi = a.xq[2 * q], eta = a.xq[2 * q + 1];
            const double x = G.x0 + G.j00 * xi + G.j01 * eta, y = G.y0 + G.j10 * xi + G.j11 * eta;
            const double wx = a.freq_pi * a.b1[mi], wy = a.freq_pi * a.b2[mi];
            if (a.kind == 0) {
                v = a.d[mi] * cos(wx * x) * cos(wy * y);
            } else {
                v = -a.d[mi] * wx * sin(wx * x) * cos(wy * y);
                vy = -a.d[mi] * wy * cos(wx * x) * sin(wy * y);
            }
        }
        if (a.kind == 0) {
            a.A[t] = v;
        } else {
            a.A[2 * t] = v;
            a.A[2 * t + 1] = vy;
        }
    }
}

// one thread per nonzero: values[mi * nnz + k] = sum over its (cell, a, b) entries
__global__ void k_gather(AArgs a, double* __restrict__ values) {
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < a.nnz; k += (int64_t)gridDim.x * blockDim.x) {
        for (int mi = 0; mi < a.nterms; ++mi) values[(size_t)mi * a.nnz + k] = 0.0;
        for (int64_t e = a.eptr[k]; e < a.eptr[k + 1]; ++e) {
            const int c = a.ecell[e];
            const int ab = a.eab[e];
            const int la = ab / a.nd, lb = ab - la * a.nd;
            const AGeo& G = a.geo[c];
            const int W = a.kind == 0 ? 1 : 2;
            // the rule in chunks of AQ points (the per-point geometric factors in registers)
            for (int q0 = 0; q0 < a.nq; q0 += AQ) {
                const int nqc = min(AQ, a.nq - q0);
                double gd[2 * AQ];
                for (int qq = 0; qq < nqc; ++qq) {
                    const int q = q0 + qq;
                    const double lam[3] = {1.0 - a.xq[2 * q] - a.xq[2 * q + 1], a.xq[2 * q], a.xq[2 * q + 1]};
                    double gr[12];
                    sgfem_fe::basis_grad(a.order, G.g, lam, gr);
                    const double wv = a.wq[q] * G.vol;
                    if (a.kind == 0) {
                        gd[qq] = wv * (gr[2 * la] * gr[2 * lb] + gr[2 * la + 1] * gr[2 * lb + 1]);
                    } else {
                        // row la tests with phi_la, column lb is the ansatz grad phi_lb
                        double v[6];
                        sgfem_fe::basis_val(a.order, lam, v);
                        gd[2 * qq] = -wv * v[la] * gr[2 * lb];
                        gd[2 * qq + 1] = -wv * v[la] * gr[2 * lb + 1];
                    }
                }
                for (int mi = 0; mi < a.nterms; ++mi) {
                    const double* Ac = a.A + ((size_t)mi * a.nc + c) * a.nq * W + (size_t)q0 * W;
                    double s = 0.0;
                    for (int q = 0; q < nqc * W; ++q) s = fma(Ac[q], gd[q], s);
                    values[(size_t)mi * a.nnz + k] += s;
                }
            }
        }
    }
}

template <typename T>
int up(sgfem_context* ctx, std::vector<void*>& own, const T* src, size_t count, T** dst) {
    void* p = nullptr;
    SG_CUDA(ctx, cudaMalloc(&p, std::max<size_t>(count, 1) * sizeof(T)));
    own.push_back(p);
    if (count) SG_CUDA(ctx, cudaMemcpyAsync(p, src, count * sizeof(T), cudaMemcpyHostToDevice, ctx->stream));
    *dst = (T*)p;
    return SGFEM_OK;
}

template <typename T>
int alloc(sgfem_context* ctx, std::vector<void*>& own, size_t count, T** dst) {
    void* p = nullptr;
    SG_CUDA(ctx, cudaMalloc(&p, std::max<size_t>(count, 1) * sizeof(T)));
    own.push_back(p);
    *dst = (T*)p;
    return SGFEM_OK;
}

struct Owned {
    std::vector<void*> p;
    ~Owned() {
        for (void* q : p) cudaFree(q);
    }
};

// origin, Jacobian, barycentric gradients and volume of every cell
int cell_geometry(sgfem_context* ctx, const sgfem_mesh* mesh, std::vector<AGeo>& geo) {
    const int64_t nc = mesh->ncells, nn = mesh->nnodes;
    geo.resize(nc);
    for (int64_t c = 0; c < nc; ++c) {
        double px[3], py[3];
        for (int k = 0; k < 3; ++k) {
            const int64_t v = mesh->cell_nodes[3 * c + k] - 1;
            if (v < 0 || v >= nn) return sg_fail(ctx, SGFEM_ERR_ARGUMENT, "cell_nodes out of range");
            px[k] = mesh->coords[2 * v];
            py[k] = mesh->coords[2 * v + 1];
        }
        AGeo& G = geo[c];
        G.x0 = px[0];
        G.y0 = py[0];
        G.j00 = px[1] - px[0];
        G.j01 = px[2] - px[0];
        G.j10 = py[1] - py[0];
        G.j11 = py[2] - py[0];
        const double det = G.j00 * G.j11 - G.j01 * G.j10;
        if (det == 0.0) return sg_fail(ctx, SGFEM_ERR_ARGUMENT, "degenerate cell");
        const double i00 = G.j11 / det, i01 = -G.j01 / det, i10 = -G.j10 / det, i11 = G.j00 / det;
        G.g[2] = i00; G.g[3] = i01;
        G.g[4] = i10; G.g[5] = i11;
        G.g[0] = -i00 - i10; G.g[1] = -i01 - i11;
        G.vol = mesh->cell_volumes[c];
    }
    return SGFEM_OK;
}

}  // namespace

namespace {

int assemble_bilinear(sgfem_context* ctx, const char* who, int kind, const sgfem_mesh* mesh,
                      const sgfem_fe_space* space, const sgfem_cosine* coef, int m0, int m1,
                      const sgfem_quadrature* quad, int64_t nnz, const int64_t* colptr, const int64_t* rowval,
                      double* values) {
    if (!ctx) return SGFEM_ERR_ARGUMENT;
    char msg[160];
    auto fail = [&](const char* what) {
        snprintf(msg, sizeof(msg), "%s: %s", who, what);
        return sg_fail(ctx, SGFEM_ERR_ARGUMENT, msg);
    };
    if (!mesh || !space || !coef || !quad || !colptr || !rowval || !values) return fail("null pointer");
    if (space->order != 1 && space->order != 2) return fail("order must be 1 or 2");
    if (m0 < 0 || m1 < m0 || m1 > coef->maxm) return fail("terms outside 0..maxm");
    if (quad->nq < 1 || quad->nq > AQMAX) return fail("cell rule must have 1..1024 points");
    const int nd = sgfem_fe::ndofs4cell(space->order);
    const int64_t nc = mesh->ncells, n = space->ndofs;
    if (nc <= 0 || n <= 0 || nnz <= 0 || colptr[n] - 1 != nnz) return fail("bad sizes");
    SG_CUDA(ctx, cudaSetDevice(ctx->device));
    // ---- cell geometry
    std::vector<AGeo> geo;
    SG_TRY(cell_geometry(ctx, mesh, geo));
    // ---- gather lists: for each CSC nonzero (row i, column j) the (cell, a, b) with
    // dof_a = i, dof_b = j, cells in increasing order (counting sort over the nonzeros)
    const size_t ne = (size_t)nc * nd * nd;
    std::vector<int64_t> pos(ne);
    std::vector<int64_t> eptr(nnz + 1, 0);
    for (int64_t c = 0; c < nc; ++c) {
        const int64_t* cd = space->cell_dofs + (size_t)nd * c;
        for (int a = 0; a < nd; ++a)
            for (int b = 0; b < nd; ++b) {
                const int64_t i = cd[a] - 1, j = cd[b] - 1;
                if (i < 0 || i >= n || j < 0 || j >= n) return sg_fail(ctx, SGFEM_ERR_ARGUMENT, "cell_dofs out of range");
                const int64_t* lo = rowval + (colptr[j] - 1);
                const int64_t* hi = rowval + (colptr[j + 1] - 1);
                const int64_t* it = std::lower_bound(lo, hi, i + 1);
                if (it == hi || *it != i + 1)
                    return sg_fail(ctx, SGFEM_ERR_ARGUMENT, "sparsity pattern misses a cell coupling");
                const int64_t k = (colptr[j] - 1) + (it - lo);
                pos[((size_t)c * nd + a) * nd + b] = k;
                eptr[k + 1]++;
            }
    }
    for (int64_t k = 0; k < nnz; ++k) eptr[k + 1] += eptr[k];
    std::vector<int64_t> fill(eptr.begin(), eptr.end() - 1);
    std::vector<int> ecell(ne);
    std::vector<unsigned char> eab(ne);
    for (int64_t c = 0; c < nc; ++c)
        for (int ab = 0; ab < nd * nd; ++ab) {
            const int64_t k = pos[(size_t)c * nd * nd + ab];
            const int64_t e = fill[k]++;
            ecell[e] = (int)c;
            eab[e] = (unsigned char)ab;
        }
    // ---- coefficient terms
    const int nterms = m1 - m0 + 1;
    std::vector<double> d(nterms, 0.0);
    std::vector<int> b1(nterms, 0), b2(nterms, 0);
    for (int mi = 0; mi < nterms; ++mi) {
        const int m = m0 + mi;
        if (m == 0) continue;
        d[mi] = coef->decay_factors[m - 1];
        b1[mi] = (int)coef->b1[m - 1];
        b2[mi] = (int)coef->b2[m - 1];
    }
    // ---- device
    Owned own;
    AArgs a{};
    a.kind = kind;
    a.order = space->order;
    a.nd = nd;
    a.nq = quad->nq;
    a.nc = (int)nc;
    a.nterms = nterms;
    a.m0 = m0;
    a.nnz = nnz;
    a.freq_pi = M_PI * coef->freq;
    a.mean = coef->mean;
    AGeo* dgeo; double *dxq, *dwq, *dd, *dA, *dval; int *db1, *db2, *dec; int64_t* dep; unsigned char* deab;
    SG_TRY(up(ctx, own.p, geo.data(), geo.size(), &dgeo));
    SG_TRY(up(ctx, own.p, quad->xref, (size_t)2 * quad->nq, &dxq));
    SG_TRY(up(ctx, own.p, quad->w, (size_t)quad->nq, &dwq));
    SG_TRY(up(ctx, own.p, d.data(), d.size(), &dd));
    SG_TRY(up(ctx, own.p, b1.data(), b1.size(), &db1));
    SG_TRY(up(ctx, own.p, b2.data(), b2.size(), &db2));
    SG_TRY(up(ctx, own.p, eptr.data(), eptr.size(), &dep));
    SG_TRY(up(ctx, own.p, ecell.data(), ecell.size(), &dec));
    SG_TRY(up(ctx, own.p, eab.data(), eab.size(), &deab));
    SG_TRY(alloc(ctx, own.p, (size_t)nterms * nc * quad->nq * (kind == 0 ? 1 : 2), &dA));
    SG_TRY(alloc(ctx, own.p, (size_t)nterms * nnz, &dval));
    a.geo = dgeo; a.xq = dxq; a.wq = dwq; a.d = dd; a.b1 = db1; a.b2 = db2; a.A = dA;
    a.eptr = dep; a.ecell = dec; a.eab = deab;
    const int grid = ctx->num_sms > 0 ? ctx->num_sms * 8 : 1216;
    k_am_qp<<<grid, 256, 0, ctx->stream>>>(a);
    SG_LAUNCHED(ctx);
    k_gather<<<grid, 256, 0, ctx->stream>>>(a, dval);
    SG_LAUNCHED(ctx);
    SG_CUDA(ctx, cudaMemcpyAsync(values, dval, (size_t)nterms * nnz * sizeof(double), cudaMemcpyDeviceToHost,
                                 ctx->stream));
    SG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return SGFEM_OK;
}

}  // namespace

extern "C" int sgfem_assemble_stiffness(sgfem_context* ctx, const sgfem_mesh* mesh, const sgfem_fe_space* space,
                                        const sgfem_cosine* coef, int m0, int m1, const sgfem_quadrature* quad,
                                        int64_t nnz, const int64_t* colptr, const int64_t* rowval, double* values) {
    return assemble_bilinear(ctx, "sgfem_assemble_stiffness", 0, mesh, space, coef, m0, m1, quad, nnz, colptr, rowval,
                             values);
}

extern "C" int sgfem_assemble_convection(sgfem_context* ctx, const sgfem_mesh* mesh, const sgfem_fe_space* space,
                                         const sgfem_cosine* coef, int m0, int m1, const sgfem_quadrature* quad,
                                         int64_t nnz, const int64_t* colptr, const int64_t* rowval, double* values) {
    return assemble_bilinear(ctx, "sgfem_assemble_convection", 1, mesh, space, coef, m0, m1, quad, nnz, colptr,
                             rowval, values);
}

// ---------------------------------------------------------------------------
// Right-hand sides b[i, k] = sum_T sum_q w_q |T| lambda_k(x_q) f(x_q) phi_i(x_q):
// lambda = 1 (P = 1) for b = (f, v) of solve!(PoissonProblemPrimal)
// (poisson_primal.jl:65-68), and the Hermite chaos coefficients of exp(factor a),
//   lambda_mu(x) = exp(sum_{m <= N} a_m(x)^2 / 2) exp(factor a_0)
//                  prod_d a_d(x)^mu_d / (sqrt(prod_d mu_d!) factor^|mu|)
// (lambda_mu of expa_PCE_mop, coefficients.jl:219-260), for the modes of
// solve!(LogTransformedPoissonProblemPrimal) (logpoisson_primal.jl:109-131).
// Device: one thread per (cell, quadrature point) evaluates w |T| f s (s the
// exponential factor) and a_1..a_M; one thread per (dof, mode) then sums its
// cells in increasing cell order (no atomics, bitwise reproducible).
namespace {

struct RArgs {
    int nd, nq, nc, M, P, ntrunc;
    int64_t n;
    const AGeo* geo;
    const double* xq;
    const double* wq;
    const double* fqp;         // nq x nc
    const double* phi;         // nq x nd: basis values at the reference points
    bool pce;
    double freq_pi, mean, factor;
    const double* d;           // decay factors of terms 1..max(M, ntrunc)
    const int* b1;
    const int* b2;
    const int* mi;             // M x P
    const double* scale;       // P: 1 / (sqrt(prod mu_d!) factor^|mu|)
    double* W;                 // nc x nq x (M + 1)
    const int64_t* dptr;       // n + 1
    const int* dcell;
    const unsigned char* dloc;
};

__global__ void k_rhs_qp(RArgs a) {
    const int W1 = a.M + 1;
    const size_t total = (size_t)a.nc * a.nq;
    for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (size_t)gridDim.x * blockDim.x) {
        const int q = (int)(t % a.nq);
        const int c = (int)(t / a.nq);
        const AGeo& G = a.geo[c];
        double* w = a.W + t * W1;
        double s = 1.0;
        if (a.pce) {
            const double xi = a.xq[2 * q], eta = a.xq[2 * q + 1];
            const double x = G.x0 + G.j00 * xi + G.j01 * eta, y = G.y0 + G.j10 * xi + G.j11 * eta;
            const int mt = a.M > a.ntrunc ? a.M : a.ntrunc;
            double sum = 0.0;
            for (int m = 1; m <= mt; ++m) {
                const double am = a.d[m - 1] * cos(a.freq_pi * a.b1[m - 1] * x) * cos(a.freq_pi * a.b2[m - 1] * y);
                if (m <= a.ntrunc) sum = fma(am, am, sum);
                if (m <= a.M) w[m] = am;
            }
            s = exp(sum / 2) * exp(a.mean * a.factor);
        }
        w[0] = a.wq[q] * G.vol * a.fqp[(size_t)c * a.nq + q] * s;
    }
}

__global__ void k_rhs_gather(RArgs a, double* __restrict__ b) {
    const int W1 = a.M + 1;
    const int64_t total = a.n * a.P;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int k = (int)(t / a.n);
        const int64_t i = t - (int64_t)k * a.n;
        const int* mu = a.mi + (size_t)k * a.M;
        double acc = 0.0;
        for (int64_t e = a.dptr[i]; e < a.dptr[i + 1]; ++e) {
            const int c = a.dcell[e], loc = a.dloc[e];
            const double* wc = a.W + (size_t)c * a.nq * W1;
            for (int q = 0; q < a.nq; ++q) {
                const double* w = wc + (size_t)q * W1;
                double lam = 1.0;
                for (int dd = 0; dd < a.M; ++dd)
                    for (int r = 0; r < mu[dd]; ++r) lam *= w[dd + 1];
                acc = fma(lam * w[0], a.phi[q * a.nd + loc], acc);
            }
        }
        b[t] = acc * a.scale[k];
    }
}

int assemble_rhs(sgfem_context* ctx, const char* who, const sgfem_mesh* mesh, const sgfem_fe_space* space,
                 const sgfem_quadrature* quad, const double* f_qp, const sgfem_cosine* coef, int64_t M, int64_t P,
                 const int32_t* multi_indices, double factor, int64_t ntrunc, double* b) {
    if (!ctx) return SGFEM_ERR_ARGUMENT;
    char msg[160];
    auto fail = [&](const char* what) {
        snprintf(msg, sizeof(msg), "%s: %s", who, what);
        return sg_fail(ctx, SGFEM_ERR_ARGUMENT, msg);
    };
    if (!mesh || !space || !quad || !f_qp || !b) return fail("null pointer");
    if (space->order != 1 && space->order != 2) return fail("order must be 1 or 2");
    if (quad->nq < 1 || quad->nq > AQMAX) return fail("cell rule must have 1..1024 points");
    const int nd = sgfem_fe::ndofs4cell(space->order);
    const int64_t nc = mesh->ncells, n = space->ndofs;
    if (nc <= 0 || n <= 0 || nc > INT32_MAX || P < 1 || M < 0) return fail("bad sizes");
    if (coef) {
        if (!multi_indices) return fail("null multi-indices");
        if (M > coef->maxm || ntrunc < 0 || ntrunc > coef->maxm) return fail("terms outside 1..maxm");
        if (factor == 0.0) return fail("factor must be nonzero");
        for (int64_t e = 0; e < M * P; ++e)
            if (multi_indices[e] < 0) return fail("negative multi-index entry");
    }
    SG_CUDA(ctx, cudaSetDevice(ctx->device));
    std::vector<AGeo> geo;
    SG_TRY(cell_geometry(ctx, mesh, geo));
    // per-dof lists of (cell, local dof), cells in increasing order
    std::vector<int64_t> dptr(n + 1, 0);
    for (int64_t e = 0; e < nc * nd; ++e) {
        const int64_t i = space->cell_dofs[e] - 1;
        if (i < 0 || i >= n) return fail("cell_dofs out of range");
        dptr[i + 1]++;
    }
    for (int64_t i = 0; i < n; ++i) dptr[i + 1] += dptr[i];
    std::vector<int64_t> fill(dptr.begin(), dptr.end() - 1);
    std::vector<int> dcell(nc * nd);
    std::vector<unsigned char> dloc(nc * nd);
    for (int64_t c = 0; c < nc; ++c)
        for (int l = 0; l < nd; ++l) {
            const int64_t e = fill[space->cell_dofs[c * nd + l] - 1]++;
            dcell[e] = (int)c;
            dloc[e] = (unsigned char)l;
        }
    std::vector<double> phi((size_t)quad->nq * nd);
    for (int q = 0; q < quad->nq; ++q) {
        const double lam[3] = {1.0 - quad->xref[2 * q] - quad->xref[2 * q + 1], quad->xref[2 * q], quad->xref[2 * q + 1]};
        sgfem_fe::basis_val(space->order, lam, phi.data() + (size_t)q * nd);
    }
    const int Mu = coef ? (int)M : 0;
    const int mt = coef ? (int)std::max(M, ntrunc) : 0;
    std::vector<double> d(std::max(mt, 1), 0.0), scale(P, 1.0);
    std::vector<int> b1(std::max(mt, 1), 0), b2(std::max(mt, 1), 0), mi(std::max<int64_t>(Mu * P, 1), 0);
    for (int m = 1; m <= mt; ++m) {
        d[m - 1] = coef->decay_factors[m - 1];
        b1[m - 1] = (int)coef->b1[m - 1];
        b2[m - 1] = (int)coef->b2[m - 1];
    }
    for (int64_t k = 0; coef && k < P; ++k) {
        double fac = 1.0, fpow = 1.0;
        for (int dd = 0; dd < Mu; ++dd) {
            const int e = multi_indices[k * M + dd];
            mi[k * Mu + dd] = e;
            for (int r = 2; r <= e; ++r) fac *= r;
            for (int r = 0; r < e; ++r) fpow *= factor;
        }
        scale[k] = 1.0 / (std::sqrt(fac) * fpow);
    }
    Owned own;
    RArgs a{};
    a.nd = nd;
    a.nq = quad->nq;
    a.nc = (int)nc;
    a.M = Mu;
    a.P = (int)P;
    a.ntrunc = coef ? (int)ntrunc : 0;
    a.n = n;
    a.pce = coef != nullptr;
    a.freq_pi = coef ? M_PI * coef->freq : 0.0;
    a.mean = coef ? coef->mean : 0.0;
    a.factor = factor;
    AGeo* dgeo; double *dxq, *dwq, *dfq, *dphi, *dd, *dsc, *dW, *db; int *db1, *db2, *dmi, *ddc; int64_t* ddp;
    unsigned char* ddl;
    SG_TRY(up(ctx, own.p, geo.data(), geo.size(), &dgeo));
    SG_TRY(up(ctx, own.p, quad->xref, (size_t)2 * quad->nq, &dxq));
    SG_TRY(up(ctx, own.p, quad->w, (size_t)quad->nq, &dwq));
    SG_TRY(up(ctx, own.p, f_qp, (size_t)quad->nq * nc, &dfq));
    SG_TRY(up(ctx, own.p, phi.data(), phi.size(), &dphi));
    SG_TRY(up(ctx, own.p, d.data(), d.size(), &dd));
    SG_TRY(up(ctx, own.p, b1.data(), b1.size(), &db1));
    SG_TRY(up(ctx, own.p, b2.data(), b2.size(), &db2));
    SG_TRY(up(ctx, own.p, mi.data(), mi.size(), &dmi));
    SG_TRY(up(ctx, own.p, scale.data(), scale.size(), &dsc));
    SG_TRY(up(ctx, own.p, dptr.data(), dptr.size(), &ddp));
    SG_TRY(up(ctx, own.p, dcell.data(), dcell.size(), &ddc));
    SG_TRY(up(ctx, own.p, dloc.data(), dloc.size(), &ddl));
    SG_TRY(alloc(ctx, own.p, (size_t)nc * quad->nq * (Mu + 1), &dW));
    SG_TRY(alloc(ctx, own.p, (size_t)n * P, &db));
    a.geo = dgeo; a.xq = dxq; a.wq = dwq; a.fqp = dfq; a.phi = dphi; a.d = dd; a.b1 = db1; a.b2 = db2;
    a.mi = dmi; a.scale = dsc; a.W = dW; a.dptr = ddp; a.dcell = ddc; a.dloc = ddl;
    const int grid = ctx->num_sms > 0 ? ctx->num_sms * 8 : 1216;
    k_rhs_qp<<<grid, 256, 0, ctx->stream>>>(a);
    SG_LAUNCHED(ctx);
    k_rhs_gather<<<grid, 256, 0, ctx->stream>>>(a, db);
    SG_LAUNCHED(ctx);
    SG_CUDA(ctx, cudaMemcpyAsync(b, db, (size_t)n * P * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    SG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return SGFEM_OK;
}

}  // namespace

extern "C" int sgfem_assemble_rhs(sgfem_context* ctx, const sgfem_mesh* mesh, const sgfem_fe_space* space,
                                  const sgfem_quadrature* quad, const double* f_qp, double* b) {
    return assemble_rhs(ctx, "sgfem_assemble_rhs", mesh, space, quad, f_qp, nullptr, 0, 1, nullptr, 1.0, 0, b);
}

extern "C" int sgfem_assemble_pce_rhs(sgfem_context* ctx, const sgfem_mesh* mesh, const sgfem_fe_space* space,
                                      const sgfem_quadrature* quad, const double* f_qp, const sgfem_cosine* coef,
                                      int64_t M, int64_t P, const int32_t* multi_indices, double factor,
                                      int64_t N_truncate, double* b) {
    if (ctx && !coef) return sg_fail(ctx, SGFEM_ERR_ARGUMENT, "sgfem_assemble_pce_rhs: null coefficient");
    return assemble_rhs(ctx, "sgfem_assemble_pce_rhs", mesh, space, quad, f_qp, coef, M, P, multi_indices, factor,
                        N_truncate, b);
}
