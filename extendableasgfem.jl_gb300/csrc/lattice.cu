// K2: the mean-based preconditioner  Z = (I (x) (a0 L)^-1) R  on sm_103a.
//
// Replaces MyPreconditionerPrimal / ldiv! (src/modelproblems/
// solvers_poisson_primal.jl:23-78), which applies LU(K_0)^-1 (K_0 with 1e60 on
// the boundary diagonals) to every mode.  When the dofs form a uniform
// lattice of the unit square (P1 or P2 on grid_unitsquare-type meshes), L is
// the 5-point Laplacian of that lattice on interior points:
//   * P1 with the diagonal split: K_0 restricted to interior rows equals
//     a0 * L exactly, so this IS the reference's preconditioner;
//   * P2: the lattice holds vertices and edge midpoints and L is the P1
//     stiffness of the once-refined mesh, spectrally equivalent to K_0 with
//     eigenvalues of L^-1 K_0 / a0 in [2/3, 4/3] for every mesh size.
// L is diagonalised by the orthonormal sine transform S (DST-I):
//   L^-1 = S diag(1 / (lam_kx + lam_ky)) S,  lam_k = 4 sin^2(pi k / (2 Nl)).
// The transform of a line of Nl-1 interior values is computed with one
// complex FFT of length Nl/2 (radix-2 decimation in frequency, bit-reversal,
// real-FFT unpacking, running sum for the odd outputs).
//
// Three passes over the SG vector (device layout: row-major dofs x modes):
//   pass X    : for each lattice row,    T = DST_x(R)
//   pass Y    : for each lattice column, T = DST_y(scale .* DST_y(T));
//               r'z = sum (DST_y T)^2 * scale  (Parseval) as block partials
//   pass X^-1 : for each lattice row,    z = DST_x(T); out = z or z + beta*out
// A CTA owns one line and 32 consecutive modes: the tile is points x 32 modes
// in shared memory, every lane works on its own mode, so each global access
// is a contiguous 32-mode segment of one dof and every shared-memory access
// is bank-conflict free.
#include "lattice_kernels.cuh"

namespace {

template <typename K>
int set_smem(sgfem_context* ctx, K kernel, size_t smem) {
    if (smem > 48 * 1024) SG_CUDA(ctx, cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    return SGFEM_OK;
}

// ---------------------------------------------------------------- Jacobi
template <typename T>
__global__ void k_jacobi(const T* __restrict__ R, T* __restrict__ out, const T* __restrict__ dinv, int n, int ld,
                         int identity, int mode, double* __restrict__ rz, const KrylovScalars* __restrict__ scal) {
    if (scal && scal->done) return;
    __shared__ double red[8];
    T beta = T(0);
    if (mode == 1 && scal && !scal->first) beta = (T)scal->beta;
    T acc_t = T(0);  // per-thread partial in the working precision
    const size_t total = (size_t)n * ld;
    for (size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total; idx += (size_t)gridDim.x * blockDim.x) {
        const int row = (int)(idx / ld);
        T d = dinv[row];
        if (identity) d = (d != T(0)) ? T(1) : T(0);
        const T r = R[idx];
        const T z = d * r;
        if (mode == 2) {
            acc_t = fma(r, z, acc_t);
        } else if (mode == 1) {
            if (d != T(0)) out[idx] = z + beta * out[idx];
        } else {
            out[idx] = z;
        }
    }
    if (mode == 2) {
        double acc = (double)acc_t;
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
        if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
        __syncthreads();
        if (threadIdx.x == 0) {
            double s = 0.0;
            for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += red[w];
            rz[blockIdx.x] = s;
        }
    }
}

}  // namespace

int sg_lattice_setup(sgfem_context* ctx) {
    const int Nl = ctx->Nl;
    if (Nl < 4 || Nl > 512 || (Nl & (Nl - 1)) != 0)
        return sg_fail(ctx, SGFEM_ERR_UNSUPPORTED, "lattice preconditioner needs a power-of-two lattice of 4..512 intervals");
    int lg = 0;
    while ((1 << lg) < Nl) ++lg;
    ctx->lat_log2 = lg;
    // smem: FP64 tile must fit
    if (lat_smem(ctx, 8) > 220 * 1024)
        return sg_fail(ctx, SGFEM_ERR_UNSUPPORTED, "lattice too large for the shared-memory line transform");
    const double pi = 3.14159265358979323846;
    const int L = Nl / 2;
    std::vector<double> tab(Nl + L + 1);
    for (int k = 0; k < L; ++k) {
        tab[k] = std::cos(2.0 * pi * k / Nl);
        tab[L + k] = std::sin(2.0 * pi * k / Nl);
    }
    for (int j = 0; j <= L; ++j) tab[Nl + j] = std::sin(pi * j / Nl);
    std::vector<float> tab32(tab.begin(), tab.end());
    const int N = Nl - 1;
    std::vector<double> lam(Nl);
    for (int k = 1; k < Nl; ++k) {
        double s = std::sin(pi * k / (2.0 * Nl));
        lam[k] = 4.0 * s * s;
    }
    // unnormalised transforms: T^2 = (Nl/2) I, so the composite carries (2/Nl)^2
    std::vector<double> sc((size_t)N * N);
    std::vector<float> sc32((size_t)N * N);
    const double a0 = ctx->lat_scale;
    const double norm = 4.0 / ((double)Nl * (double)Nl);
    for (int kx = 1; kx < Nl; ++kx)
        for (int ky = 1; ky < Nl; ++ky) {
            double v = norm / (a0 * (lam[kx] + lam[ky]));
            sc[(size_t)(kx - 1) * N + (ky - 1)] = v;
            sc32[(size_t)(kx - 1) * N + (ky - 1)] = (float)v;
        }
    SG_CUDA(ctx, cudaMalloc(&ctx->d_lat_tab64, tab.size() * sizeof(double)));
    SG_CUDA(ctx, cudaMemcpy(ctx->d_lat_tab64, tab.data(), tab.size() * sizeof(double), cudaMemcpyHostToDevice));
    SG_CUDA(ctx, cudaMalloc(&ctx->d_lat_tab32, tab32.size() * sizeof(float)));
    SG_CUDA(ctx, cudaMemcpy(ctx->d_lat_tab32, tab32.data(), tab32.size() * sizeof(float), cudaMemcpyHostToDevice));
    SG_CUDA(ctx, cudaMalloc(&ctx->d_lat_scale64, sc.size() * sizeof(double)));
    SG_CUDA(ctx, cudaMemcpy(ctx->d_lat_scale64, sc.data(), sc.size() * sizeof(double), cudaMemcpyHostToDevice));
    SG_CUDA(ctx, cudaMalloc(&ctx->d_lat_scale32, sc32.size() * sizeof(float)));
    SG_CUDA(ctx, cudaMemcpy(ctx->d_lat_scale32, sc32.data(), sc32.size() * sizeof(float), cudaMemcpyHostToDevice));
    return SGFEM_OK;
}

namespace {

template <typename T>
sglat::PassXFn<T> pass_x_fn(int LGL);
template <typename T>
sglat::PassYFn<T> pass_y_fn(int LGL);
template <typename T>
sglat::PassYFn<T> pass_yb_fn(int LGL);
template <>
sglat::PassXFn<float> pass_x_fn<float>(int LGL) { return local_pass_x_fn<float>(LGL); }
template <>
sglat::PassYFn<float> pass_y_fn<float>(int LGL) { return local_pass_y_fn<float>(LGL); }
template <>
sglat::PassYFn<float> pass_yb_fn<float>(int LGL) { return local_pass_yb_fn<float>(LGL); }
template <>
sglat::PassXFn<double> pass_x_fn<double>(int LGL) { return sglat::pass_x_fn_f64(LGL); }
template <>
sglat::PassYFn<double> pass_y_fn<double>(int LGL) { return sglat::pass_y_fn_f64(LGL); }
template <>
sglat::PassYFn<double> pass_yb_fn<double>(int LGL) { return sglat::pass_yb_fn_f64(LGL); }

template <typename T>
int launch_x(sgfem_context* ctx, const void* in, void* out, const T* tab, int mode, const KrylovScalars* scal) {
    LatGeom g = geom(ctx);
    g.async = ((uintptr_t)in % 16) == 0;
    sglat::PassXFn<T> fn = pass_x_fn<T>(ctx->lat_log2 - 1);
    if (!fn) return sg_fail(ctx, SGFEM_ERR_UNSUPPORTED, "lattice size outside the compiled range");
    const int grid = (g.Nl - 1) * g.nchunk;
    fn<<<grid, LAT_THREADS, lat_smem(ctx, sizeof(T)), ctx->stream>>>((const T*)in, (T*)out, tab, g, mode, scal);
    SG_LAUNCHED(ctx);
    return SGFEM_OK;
}

template <typename T>
int launch_y(sgfem_context* ctx, void* buf, const T* tab, const T* scale, double* rz, int* nblocks,
             const KrylovScalars* scal) {
    LatGeom g = geom(ctx);
    g.async = ((uintptr_t)buf % 16) == 0;
    sglat::PassYFn<T> fn = ctx->lat_block ? pass_yb_fn<T>(ctx->lat_log2 - 1) : pass_y_fn<T>(ctx->lat_log2 - 1);
    if (!fn) return sg_fail(ctx, SGFEM_ERR_UNSUPPORTED, "lattice size outside the compiled range");
    const int grid = ctx->lat_block ? (g.Nl / 2) * (int)((g.ld + 15) / 16) : (g.Nl - 1) * g.nchunk;
    if (nblocks) *nblocks = grid;
    fn<<<grid, LAT_THREADS, lat_smem(ctx, sizeof(T)), ctx->stream>>>((T*)buf, tab, scale, g, rz, scal);
    SG_LAUNCHED(ctx);
    return SGFEM_OK;
}

}  // namespace

int sg_lattice_configure(sgfem_context* ctx) {
    const int LGL = ctx->lat_log2 - 1;
    if (!pass_x_fn<double>(LGL)) return sg_fail(ctx, SGFEM_ERR_UNSUPPORTED, "lattice size outside the compiled range");
    SG_TRY(set_smem(ctx, pass_x_fn<double>(LGL), lat_smem(ctx, 8)));
    SG_TRY(set_smem(ctx, pass_y_fn<double>(LGL), lat_smem(ctx, 8)));
    SG_TRY(set_smem(ctx, pass_x_fn<float>(LGL), lat_smem(ctx, 4)));
    SG_TRY(set_smem(ctx, pass_y_fn<float>(LGL), lat_smem(ctx, 4)));
    SG_TRY(set_smem(ctx, pass_yb_fn<double>(LGL), lat_smem(ctx, 8)));
    SG_TRY(set_smem(ctx, pass_yb_fn<float>(LGL), lat_smem(ctx, 4)));
    return SGFEM_OK;
}

int sg_lat_max_blocks(const sgfem_context* ctx) {
    if (!ctx->lattice) return 1;
    return std::max((ctx->Nl - 1) * (int)((ctx->ld + 31) / 32), (ctx->Nl / 2) * (int)((ctx->ld + 15) / 16));
}

int sg_lat_pass_x(sgfem_context* ctx, int precision, const void* R, void* T, const KrylovScalars* scal) {
    if (precision == SGFEM_FP64) return launch_x<double>(ctx, R, T, ctx->d_lat_tab64, 0, scal);
    return launch_x<float>(ctx, R, T, ctx->d_lat_tab32, 0, scal);
}

int sg_lat_pass_y(sgfem_context* ctx, int precision, void* T, double* rz, int* nblocks, const KrylovScalars* scal) {
    if (precision == SGFEM_FP64)
        return launch_y<double>(ctx, T, ctx->d_lat_tab64, ctx->lat_block ? ctx->d_lat_blk64 : ctx->d_lat_scale64, rz,
                                nblocks, scal);
    return launch_y<float>(ctx, T, ctx->d_lat_tab32, ctx->lat_block ? ctx->d_lat_blk32 : ctx->d_lat_scale32, rz,
                           nblocks, scal);
}

// Exact mean preconditioner for lattice operators.  Every interior row of class
// c = (x % 2, y % 2) must carry the same stencil w_c(d), |d| <= 2, on the interior
// points (P1 and P2 Lagrange elements on the uniform triangulation with a constant
// mean coefficient); then the orthonormal 2-D sine transform S maps K_0 (interior
// rows and columns) to 4x4 blocks on the frequencies {i, Nl-i} x {j, Nl-j}:
//   B_ab = <phi_a, K_0 phi_b> = sum_c sum_d w_c(d) X_c,dx(a_x, b_x) Y_c,dy(a_y, b_y),
//   X_c,dx(k, l) = sum_{x = c_x mod 2, 1 <= x, x + dx <= Nl - 1} s_k(x) s_l(x + dx),
// s_k(x) = sqrt(2/Nl) sin(pi k x / Nl).  The table holds (2/Nl)^2 B^-1 (upper
// triangle, frequency pairs that collapse for i or j = Nl/2 left out), so that
// pass Y applies K_0^-1 = (2/Nl)^2 T B^-1 T with the unnormalised transforms T.
// This is the reference's LU(K_0) solve (solvers_poisson_primal.jl:23-78) on
// interior rows.  Anything else keeps the 5-point Laplacian scaled by the mean.
int sg_lattice_blocks(sgfem_context* ctx, const std::vector<int64_t>& rowptr, const std::vector<int32_t>& col,
                      const std::vector<double>& val64) {
    ctx->lat_block = false;
    const int Nl = ctx->Nl, np = Nl + 1, M1 = ctx->M1;
    constexpr int R = 2;
    const char* ev = getenv("SGFEM_LAT_BLOCK");
    if (ev && atoi(ev) == 0) {
        ctx->lat_log = "5-point Laplacian (SGFEM_LAT_BLOCK=0)";
        return SGFEM_OK;
    }
    if (Nl < 8 || !ctx->lat_order || ctx->win_hx > R || ctx->win_hy > R) {
        ctx->lat_log = "5-point Laplacian (lattice too small or couplings too long for the block form)";
        return SGFEM_OK;
    }
    auto boundary = [&](int x, int y) { return x == 0 || y == 0 || x == Nl || y == Nl; };
    for (int64_t r = 0; r < (int64_t)np * np; ++r)
        if ((ctx->bmask_host[r] != 0) != boundary((int)(r % np), (int)(r / np))) {
            ctx->lat_log = "5-point Laplacian (Dirichlet dofs are not the lattice boundary)";
            return SGFEM_OK;
        }
    auto value = [&](int64_t r, int32_t c) -> double {
        auto b = col.begin() + rowptr[r], e = col.begin() + rowptr[r + 1];
        auto it = std::lower_bound(b, e, c);
        return (it != e && *it == c) ? val64[(size_t)(it - col.begin()) * M1] : 0.0;
    };
    double w[2][2][2 * R + 1][2 * R + 1];
    double wmax = 0.0;
    for (int cy = 0; cy < 2; ++cy)
        for (int cx = 0; cx < 2; ++cx) {
            const int x0 = Nl / 2 + cx, y0 = Nl / 2 + cy;
            for (int dy = -R; dy <= R; ++dy)
                for (int dx = -R; dx <= R; ++dx) {
                    const double v = value((int64_t)y0 * np + x0, (y0 + dy) * np + x0 + dx);
                    w[cy][cx][dy + R][dx + R] = v;
                    wmax = std::max(wmax, std::fabs(v));
                }
        }
    const double tol = 1e-11 * wmax;
    for (int y = 1; y < Nl; ++y)
        for (int x = 1; x < Nl; ++x) {
            const int64_t r = (int64_t)y * np + x;
            const int cx = x & 1, cy = y & 1;
            double seen = 0.0, want = 0.0;
            for (int64_t k = rowptr[r]; k < rowptr[r + 1]; ++k) {
                const int jx = col[k] % np, jy = col[k] / np;
                if (boundary(jx, jy)) continue;
                const int dx = jx - x, dy = jy - y;
                const double v = val64[(size_t)k * M1];
                if (std::abs(dx) > R || std::abs(dy) > R || std::fabs(v - w[cy][cx][dy + R][dx + R]) > tol) {
                    ctx->lat_log = "5-point Laplacian (K_0 is not translation invariant on the lattice)";
                    return SGFEM_OK;
                }
                seen += std::fabs(v);
            }
            for (int dy = -R; dy <= R; ++dy)
                for (int dx = -R; dx <= R; ++dx)
                    if (!boundary(x + dx, y + dy) && x + dx >= 0 && y + dy >= 0 && x + dx <= Nl && y + dy <= Nl)
                        want += std::fabs(w[cy][cx][dy + R][dx + R]);
            if (std::fabs(seen - want) > 1e-10 * want) {
                ctx->lat_log = "5-point Laplacian (K_0 is not translation invariant on the lattice)";
                return SGFEM_OK;
            }
        }
    // one-dimensional sums X_c,d(a, b) for the frequency pair (i, Nl - i), i = 1..H
    const int H = Nl / 2;
    const double pi = 3.14159265358979323846;
    std::vector<double> sn(2 * Nl);
    for (int m = 0; m < 2 * Nl; ++m) sn[m] = std::sqrt(2.0 / Nl) * std::sin(pi * m / Nl);
    auto sv = [&](int k, int x) { return sn[(size_t)((int64_t)k * x % (2 * Nl))]; };
    std::vector<double> A((size_t)(H + 1) * 2 * (2 * R + 1) * 4, 0.0);
    auto aidx = [&](int i, int c, int d, int a, int b) { return ((((size_t)i * 2 + c) * (2 * R + 1) + d + R) * 2 + a) * 2 + b; };
    for (int i = 1; i <= H; ++i) {
        const int f[2] = {i, Nl - i};
        for (int c = 0; c < 2; ++c)
            for (int d = -R; d <= R; ++d)
                for (int a = 0; a < 2; ++a)
                    for (int b = 0; b < 2; ++b) {
                        double sum = 0.0;
                        for (int x = c; x < Nl; x += 2)
                            if (x >= 1 && x + d >= 1 && x + d <= Nl - 1) sum += sv(f[a], x) * sv(f[b], x + d);
                        A[aidx(i, c, d, a, b)] = sum;
                    }
    }
    const double norm = 4.0 / ((double)Nl * (double)Nl);
    std::vector<double> blk((size_t)H * H * 10);
    for (int i = 1; i <= H; ++i)
        for (int j = 1; j <= H; ++j) {
            double B[4][4] = {};
            for (int cy = 0; cy < 2; ++cy)
                for (int cx = 0; cx < 2; ++cx)
                    for (int dy = -R; dy <= R; ++dy)
                        for (int dx = -R; dx <= R; ++dx) {
                            const double wv = w[cy][cx][dy + R][dx + R];
                            if (wv == 0.0) continue;
                            for (int a = 0; a < 4; ++a)
                                for (int b = 0; b < 4; ++b)
                                    B[a][b] += wv * A[aidx(i, cx, dx, a & 1, b & 1)] * A[aidx(j, cy, dy, a >> 1, b >> 1)];
                        }
            // distinct frequencies: index a = 2 ay + ax, ax < nx, ay < ny
            const int nx = (i == H) ? 1 : 2, ny = (j == H) ? 1 : 2;
            int id[4], k = 0;
            for (int ay = 0; ay < ny; ++ay)
                for (int ax = 0; ax < nx; ++ax) id[k++] = 2 * ay + ax;
            // Gauss-Jordan inverse of the k x k block (symmetric positive definite)
            double Mx[4][8] = {};
            for (int r = 0; r < k; ++r) {
                for (int c = 0; c < k; ++c) Mx[r][c] = B[id[r]][id[c]];
                Mx[r][k + r] = 1.0;
            }
            for (int c = 0; c < k; ++c) {
                int pr = c;
                for (int r = c + 1; r < k; ++r)
                    if (std::fabs(Mx[r][c]) > std::fabs(Mx[pr][c])) pr = r;
                if (!(std::fabs(Mx[pr][c]) > 1e-14 * wmax)) {
                    ctx->lat_log = "5-point Laplacian (singular sine-transform block)";
                    return SGFEM_OK;
                }
                for (int t = 0; t < 2 * k; ++t) std::swap(Mx[c][t], Mx[pr][t]);
                const double piv = Mx[c][c];
                for (int t = 0; t < 2 * k; ++t) Mx[c][t] /= piv;
                for (int r = 0; r < k; ++r)
                    if (r != c) {
                        const double f = Mx[r][c];
                        for (int t = 0; t < 2 * k; ++t) Mx[r][t] -= f * Mx[c][t];
                    }
            }
            double Bi[4][4] = {};
            for (int r = 0; r < k; ++r)
                for (int c = 0; c < k; ++c) Bi[id[r]][id[c]] = norm * 0.5 * (Mx[r][k + c] + Mx[c][k + r]);
            for (int r = 0; r < 4; ++r)
                if (Bi[r][r] < 0.0) {
                    ctx->lat_log = "5-point Laplacian (sine-transform block not positive definite)";
                    return SGFEM_OK;
                }
            double* o = &blk[((size_t)(i - 1) * H + (j - 1)) * 10];
            o[0] = Bi[0][0]; o[1] = Bi[0][1]; o[2] = Bi[0][2]; o[3] = Bi[0][3];
            o[4] = Bi[1][1]; o[5] = Bi[1][2]; o[6] = Bi[1][3];
            o[7] = Bi[2][2]; o[8] = Bi[2][3];
            o[9] = Bi[3][3];
        }
    std::vector<float> blk32(blk.begin(), blk.end());
    SG_CUDA(ctx, cudaMalloc(&ctx->d_lat_blk64, blk.size() * sizeof(double)));
    SG_CUDA(ctx, cudaMemcpy(ctx->d_lat_blk64, blk.data(), blk.size() * sizeof(double), cudaMemcpyHostToDevice));
    SG_CUDA(ctx, cudaMalloc(&ctx->d_lat_blk32, blk32.size() * sizeof(float)));
    SG_CUDA(ctx, cudaMemcpy(ctx->d_lat_blk32, blk32.data(), blk32.size() * sizeof(float), cudaMemcpyHostToDevice));
    ctx->lat_block = true;
    ctx->lat_log = "exact K_0^-1: 4x4 blocks of the 2-D sine transform";
    return SGFEM_OK;
}

int sg_lat_pass_xinv(sgfem_context* ctx, int precision, const void* T, void* out, int mode, const KrylovScalars* scal) {
    if (precision == SGFEM_FP64) return launch_x<double>(ctx, T, out, ctx->d_lat_tab64, mode, scal);
    return launch_x<float>(ctx, T, out, ctx->d_lat_tab32, mode, scal);
}

int sg_jacobi(sgfem_context* ctx, int precision, const void* R, void* out, int mode, int identity, double* rz,
              int* nblocks, const KrylovScalars* scal) {
    const int threads = 256;
    int grid = (int)std::min<int64_t>(((int64_t)ctx->n * ctx->ld + threads - 1) / threads, (int64_t)ctx->num_sms * 8);
    if (grid < 1) grid = 1;
    if (nblocks) *nblocks = grid;
    if (precision == SGFEM_FP64)
        k_jacobi<double><<<grid, threads, 0, ctx->stream>>>((const double*)R, (double*)out, ctx->d_dinv64, (int)ctx->n,
                                                            (int)ctx->ld, identity, mode, rz, scal);
    else
        k_jacobi<float><<<grid, threads, 0, ctx->stream>>>((const float*)R, (float*)out, ctx->d_dinv32, (int)ctx->n,
                                                           (int)ctx->ld, identity, mode, rz, scal);
    SG_LAUNCHED(ctx);
    return SGFEM_OK;
}
