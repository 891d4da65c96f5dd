// Stiffness matrices of the affine cosine coefficient, assembled on the GPU.
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
#include <cmath>
#include <vector>

#include "fe_basis.cuh"
#include "sgfem_internal.h"

namespace {

constexpr int AQ = 16;  // largest cell rule

struct AGeo {
    double x0, y0, j00, j10, j01, j11, g[6], vol;
};

struct AArgs {
    int order, nd, nq, nc, nterms, m0;
    int64_t nnz;
    const AGeo* geo;
    const double* xq;    // 2 x nq
    const double* wq;
    double freq_pi, mean;
    const double* d;     // d[m - m0] (d of m = 0 unused)
    const int* b1;
    const int* b2;
    double* A;           // nterms x nc x nq: a_m at the quadrature points
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
        double v = a.mean;
        if (m > 0) {
            const AGeo& G = a.geo[c];
            const double xi = a.xq[2 * q], eta = a.xq[2 * q + 1];
            const double x = G.x0 + G.j00 * xi + G.j01 * eta, y = G.y0 + G.j10 * xi + G.j11 * eta;
            v = a.d[mi] * cos(a.freq_pi * a.b1[mi] * x) * cos(a.freq_pi * a.b2[mi] * y);
        }
        a.A[t] = v;
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
            double gd[AQ];
            for (int q = 0; q < a.nq; ++q) {
                const double lam[3] = {1.0 - a.xq[2 * q] - a.xq[2 * q + 1], a.xq[2 * q], a.xq[2 * q + 1]};
                double gr[12];
                sgfem_fe::basis_grad(a.order, G.g, lam, gr);
                gd[q] = a.wq[q] * G.vol * (gr[2 * la] * gr[2 * lb] + gr[2 * la + 1] * gr[2 * lb + 1]);
            }
            for (int mi = 0; mi < a.nterms; ++mi) {
                const double* Ac = a.A + ((size_t)mi * a.nc + c) * a.nq;
                double s = 0.0;
                for (int q = 0; q < a.nq; ++q) s = fma(Ac[q], gd[q], s);
                values[(size_t)mi * a.nnz + k] += s;
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

}  // namespace

extern "C" int sgfem_assemble_stiffness(sgfem_context* ctx, const sgfem_mesh* mesh, const sgfem_fe_space* space,
                                        const sgfem_cosine* coef, int m0, int m1, const sgfem_quadrature* quad,
                                        int64_t nnz, const int64_t* colptr, const int64_t* rowval, double* values) {
    if (!ctx) return SGFEM_ERR_ARGUMENT;
    if (!mesh || !space || !coef || !quad || !colptr || !rowval || !values)
        return sg_fail(ctx, SGFEM_ERR_ARGUMENT, "sgfem_assemble_stiffness: null pointer");
    if (space->order != 1 && space->order != 2)
        return sg_fail(ctx, SGFEM_ERR_ARGUMENT, "sgfem_assemble_stiffness: order must be 1 or 2");
    if (m0 < 0 || m1 < m0 || m1 > coef->maxm)
        return sg_fail(ctx, SGFEM_ERR_ARGUMENT, "sgfem_assemble_stiffness: terms outside 0..maxm");
    if (quad->nq < 1 || quad->nq > AQ) return sg_fail(ctx, SGFEM_ERR_ARGUMENT, "cell rule must have 1..16 points");
    const int nd = sgfem_fe::ndofs4cell(space->order);
    const int64_t nc = mesh->ncells, nn = mesh->nnodes, n = space->ndofs;
    if (nc <= 0 || n <= 0 || nnz <= 0 || colptr[n] - 1 != nnz)
        return sg_fail(ctx, SGFEM_ERR_ARGUMENT, "sgfem_assemble_stiffness: bad sizes");
    SG_CUDA(ctx, cudaSetDevice(ctx->device));
    // ---- cell geometry
    std::vector<AGeo> geo(nc);
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
    SG_TRY(alloc(ctx, own.p, (size_t)nterms * nc * quad->nq, &dA));
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
