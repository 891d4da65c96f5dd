/*
 * Oracle / CPU baseline: plain-C restatement of the reference operator apply.
 *
 * TEST INFRASTRUCTURE ONLY (see oracle/__init__.py): used by tests as a
 * checker and by bench.py as the timed CPU baseline, never by the product.
 *
 * Follows mul!(Ax, S::MySystemPrimal, x) in
 * src/modelproblems/solvers_poisson_primal.jl:86-124 of ExtendableASGFEM.jl
 * step by step: for every mode mu, Ax_mu = K_0 x_mu, then for every (nu, e)
 * with g = G[(e-1)P + mu, nu] != 0 one full sparse matrix-vector product
 * Ax_mu += g * K_e x_nu (addblock_matmul! over the CSC storage), then the
 * Dirichlet rows of Ax_mu are zeroed.  Matrices are CSC (0-based here), G is
 * dense (M*P) x P row-major, vectors are the column-major n x P SGFEVector
 * entries.  The loop over mu is independent per mode; with OpenMP it is
 * split across host threads (nthreads > 1), else it runs single-threaded like
 * the reference.
 */
#include <stdint.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

static void csc_matvec_add(int64_t n, const int64_t* colptr, const int64_t* rowval, const double* nzval,
                           const double* x, double* y, double factor) {
    for (int64_t col = 0; col < n; ++col) {
        const double xc = x[col];
        for (int64_t r = colptr[col]; r < colptr[col + 1]; ++r) y[rowval[r]] += nzval[r] * xc * factor;
    }
}

/* mats: M+1 CSC matrices given by arrays of pointers */
void oracle_sg_mul(int64_t n, int64_t P, int64_t M, const int64_t* const* colptr, const int64_t* const* rowval,
                   const double* const* nzval, const double* G, int64_t nb, const int64_t* bdofs, const double* x,
                   double* Ax, int nthreads) {
    memset(Ax, 0, sizeof(double) * (size_t)(n * P));
#ifdef _OPENMP
    if (nthreads < 1) nthreads = 1;
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads)
#endif
    for (int64_t mu = 0; mu < P; ++mu) {
        double* y = Ax + mu * n;
        csc_matvec_add(n, colptr[0], rowval[0], nzval[0], x + mu * n, y, 1.0);
        for (int64_t nu = 0; nu < P; ++nu) {
            for (int64_t e = 1; e <= M; ++e) {
                const double g = G[((e - 1) * P + mu) * P + nu];
                if (g != 0.0) csc_matvec_add(n, colptr[e], rowval[e], nzval[e], x + nu * n, y, g);
            }
        }
        for (int64_t k = 0; k < nb; ++k) y[bdofs[k]] = 0.0;
    }
}

int oracle_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
