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
#include <stdlib.h>
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

/*
 * ldiv!(y, P, b) of solvers_poisson_primal.jl:47-78 with the LU factors of
 * K_0 (1e60 on the boundary diagonals) computed once by SuperLU:
 * Pr A Pc = L U, L unit lower and U upper triangular, both CSC (0-based,
 * int64 indices), perm_r / perm_c as returned by SciPy's splu
 * (Pr[perm_r[i], i] = 1, Pc[i, perm_c[i]] = 1, so x = Pc U^-1 L^-1 Pr b).  Every mode mu of the
 * column-major n x P block B is solved independently, as the reference does
 * one LU solve per mode; with OpenMP the modes are split over host threads in
 * groups of RB right-hand sides that share one pass over the factors.
 */
#define RB 8
void oracle_lu_solve_modes(int64_t n, int64_t P, const int64_t* Lp, const int64_t* Li, const double* Lx,
                           const int64_t* Up, const int64_t* Ui, const double* Ux, const int64_t* perm_r,
                           const int64_t* perm_c, const double* B, double* X, int nthreads) {
    const int64_t ngroups = (P + RB - 1) / RB;
#ifdef _OPENMP
    if (nthreads < 1) nthreads = 1;
#pragma omp parallel num_threads(nthreads)
#endif
    {
        double* w = (double*)malloc(sizeof(double) * (size_t)n * RB);
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 1)
#endif
        for (int64_t g = 0; g < ngroups; ++g) {
            const int64_t m0 = g * RB;
            const int64_t nr = (P - m0 < RB) ? (P - m0) : RB;
            /* w = Pr b, interleaved [row][rhs] */
            for (int64_t r = 0; r < nr; ++r) {
                const double* b = B + (m0 + r) * n;
                for (int64_t i = 0; i < n; ++i) w[perm_r[i] * RB + r] = b[i];
            }
            /* L z = w (unit diagonal; the diagonal entry of each column is skipped) */
            for (int64_t j = 0; j < n; ++j) {
                double* wj = w + j * RB;
                for (int64_t p = Lp[j]; p < Lp[j + 1]; ++p) {
                    const int64_t i = Li[p];
                    if (i <= j) continue;
                    const double l = Lx[p];
                    double* wi = w + i * RB;
                    for (int64_t r = 0; r < nr; ++r) wi[r] -= l * wj[r];
                }
            }
            /* U v = z (column-oriented back substitution) */
            for (int64_t j = n - 1; j >= 0; --j) {
                double* wj = w + j * RB;
                double d = 0.0;
                for (int64_t p = Up[j]; p < Up[j + 1]; ++p)
                    if (Ui[p] == j) d = Ux[p];
                for (int64_t r = 0; r < nr; ++r) wj[r] /= d;
                for (int64_t p = Up[j]; p < Up[j + 1]; ++p) {
                    const int64_t i = Ui[p];
                    if (i >= j) continue;
                    const double u = Ux[p];
                    double* wi = w + i * RB;
                    for (int64_t r = 0; r < nr; ++r) wi[r] -= u * wj[r];
                }
            }
            /* x = Pc v */
            for (int64_t r = 0; r < nr; ++r) {
                double* x = X + (m0 + r) * n;
                for (int64_t i = 0; i < n; ++i) x[i] = w[perm_c[i] * RB + r];
            }
        }
        free(w);
    }
}

/* BLAS-1 helpers of the Krylov loop (Krylov.jl calls BLAS dot / axpy) */
double oracle_dot(int64_t n, const double* x, const double* y, int nthreads) {
    double s = 0.0;
#ifdef _OPENMP
    if (nthreads < 1) nthreads = 1;
#pragma omp parallel for reduction(+ : s) schedule(static) num_threads(nthreads)
#endif
    for (int64_t i = 0; i < n; ++i) s += x[i] * y[i];
    return s;
}

void oracle_axpy(int64_t n, double a, const double* x, double* y, int nthreads) {
#ifdef _OPENMP
    if (nthreads < 1) nthreads = 1;
#pragma omp parallel for schedule(static) num_threads(nthreads)
#endif
    for (int64_t i = 0; i < n; ++i) y[i] += a * x[i];
}

void oracle_scale_copy(int64_t n, double a, const double* x, double* y, int nthreads) {
#ifdef _OPENMP
    if (nthreads < 1) nthreads = 1;
#pragma omp parallel for schedule(static) num_threads(nthreads)
#endif
    for (int64_t i = 0; i < n; ++i) y[i] = a * x[i];
}
