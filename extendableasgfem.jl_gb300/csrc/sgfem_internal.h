// Internal declarations of the sm_103a stochastic-Galerkin library (libsgfem).
//
// Device data layout (all in HBM, owned by the context):
//   * SG vectors: n rows (device dof order) x ld columns, row-major, ld = P
//     rounded up to a multiple of 4; padding columns are kept at zero.  One
//     CSR nonzero (i, j) thus gathers the contiguous mode vector of dof j.
//   * spatial operators: one CSR pattern (union of the K_m patterns, int32
//     rowptr / colidx) with the M+1 values of a nonzero stored contiguously,
//     vals[nz * M1 + m], in FP64 and in FP32.
//   * coupling: the pair list Q = {(0, nu)} u {(m, nu) : G_m column nu != 0}
//     and, per output mode mu, the list of (g, q) with g = G_m[mu, nu].
// The device dof order is the lattice order (row by row) when the dof
// coordinates form a uniform lattice of the unit square, else the caller's.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/sgfem.h"

struct HostCSC {
    int64_t n = 0;
    std::vector<int64_t> colptr;  // 0-based
    std::vector<int64_t> rowval;  // 0-based
    std::vector<double> nzval;
    bool set = false;
};

// scalars of a Krylov solve kept on the device (no host round trip per iteration)
struct KrylovScalars {
    double rho;      // r'z of the current iterate
    double pq;       // p'Ap
    double alpha;
    double beta;
    double rr;       // ||r||^2
    double tol2;     // stop when rr <= tol2
    int done;        // 1 once converged or failed; kernels return early
    int status;      // SGFEM_OK / SGFEM_ERR_BREAKDOWN / SGFEM_ERR_NONFINITE
    int iters;       // iterations completed
    int first;       // 1 before the first preconditioner application (beta = 0)
    int maxit;       // iteration cap of the current PCG run
    int loops;       // device-loop bodies run by the current PCG run
};

struct DeviceBuf {
    void* p = nullptr;
    size_t bytes = 0;
};

enum { SG_NBUF = 14 };

struct MeanChol;  // sparse-Cholesky mean preconditioner (meanchol.cu)
struct SmallPCG;  // one-cluster FP32 PCG for small lattice problems (small.cu)

struct sgfem_context {
    int device = 0;
    cudaStream_t stream = nullptr;
    std::string err;
    int num_sms = 0;

    // ---- host-side setup state ----
    int64_t n = -1;          // spatial dofs
    int64_t P = -1;          // modes
    int64_t M = -1;          // number of K_m beyond K_0
    std::vector<HostCSC> mats;
    std::vector<int64_t> G_colptr, G_rowval;
    std::vector<double> G_val;
    bool has_G = false;
    bool batched = false;        // block-diagonal sample operator (sgfem_set_samples)
    std::vector<double> ysamp;   // M x S
    double* d_y64 = nullptr;     // [S][M1] coefficients, y_{s,0} = 1
    float* d_y32 = nullptr;
    double* d_kval64 = nullptr;  // [nnz][ld]: K(y_s) = sum_m y_{s,m} K_m per sample (nullptr: combined on the fly)
    float* d_kval32 = nullptr;
    DeviceBuf w_valhl;           // K_m values as (hi, lo) float pairs for the double-FP32 combination
    DeviceBuf w_yhl;             // sample coefficients as (hi, lo) float pairs
    DeviceBuf w_samp;            // arrays of the last sgfem_evaluate_samples / sgfem_sampling_error
    bool samples_x_valid = false;  // w_vec[10] holds the solutions of the current samples
    int sampling_form = 0;         // last sgfem_sampling_error: 0 none, 1 quadratic forms, 2 quadrature points
    std::vector<int64_t> bdofs;  // 0-based caller numbering
    bool has_bdofs = false;
    std::vector<double> dof_xy;  // 2 x n column-major
    bool finalized = false;

    // ---- device-side structures ----
    int64_t ld = 0;            // row stride of device SG vectors
    int64_t nnz = 0;
    int M1 = 0;                // M + 1
    std::vector<int32_t> perm;   // device row -> caller dof
    std::vector<int32_t> iperm;  // caller dof -> device row
    int* d_rowptr = nullptr;
    int* d_col = nullptr;
    double* d_val64 = nullptr;
    float* d_val32 = nullptr;
    unsigned char* d_bmask = nullptr;
    int* d_iperm = nullptr;    // caller dof -> device row
    std::vector<unsigned char> bmask_host;
    double* d_dinv64 = nullptr;  // 1/diag(K_0), 0 on boundary rows (Jacobi)
    float* d_dinv32 = nullptr;

    // coupling schedule
    int Qn = 0;
    int* d_qtab = nullptr;         // packed (m << 16) | nu, length Qn
    int* d_combptr = nullptr;      // P + 1
    int* d_combq = nullptr;
    double* d_combg64 = nullptr;
    float* d_combg32 = nullptr;
    int ncomb = 0;
    float2* d_valdf = nullptr;     // K_m values as (hi, lo) float pairs (double-FP32 residual)
    float2* d_combgdf = nullptr;   // G combination coefficients as (hi, lo)

    // host copies of the pair list and the per-column combination lists (device columns)
    std::vector<int32_t> h_qtab, h_combptr, h_combq;
    std::vector<double> h_combg;
    struct SplitApply* split = nullptr;  // split-slot form of the specialised FP32 apply (jit_split.cu)
    int jit_split_req = 1;               // asked for (SGFEM_JIT_SPLIT)
    int jit_split = 0;                   // in use
    int row_nnz_max = -1;                // longest row of the union pattern (set at finalize)

    // device column order of the modes
    std::vector<int32_t> mode_of_col;  // device column -> caller mode
    std::vector<int32_t> imode;        // caller mode -> device column
    int* d_mode_of_col = nullptr;

    // specialised FP32 apply (NVRTC): slots (KLE pair, 32-column group)
    int M1P = 0;                            // value stride of d_val32p (M+1 rounded up to 4)
    float* d_val32p = nullptr;              // [nnz][M1P]
    std::vector<int> jit_slot_of;           // [pair * KG + group] -> slot or -1
    std::vector<std::pair<int, int>> jit_slots;  // (pair, group)
    int* d_jptr = nullptr;                  // P + 1
    int* d_joff = nullptr;                  // accumulator offsets
    float* d_jg = nullptr;                  // coefficients
    int2* d_jtab = nullptr;                 // lane schedule of the combination, [T][32]
    int jit_T = 0;                          // entries per lane in d_jtab (-1: does not fit)
    int jit_np_req = 1;                     // passes asked for (SGFEM_JIT_PASSES)
    int jit_np = 1;                         // passes over the nonzeros of a row (column-group ranges)
    std::vector<int> jit_pass_k0;           // first column group of pass p (np + 1 entries)
    std::vector<int> jit_pass_slot0;        // first slot of pass p (np + 1 entries)
    std::vector<int> jit_pass_T;            // combination entries per lane of pass p
    int jit_rchunk = 8;                     // rows per warp chunk
    int jit_prefetch = 0;
    int jit_pfd = 1;                        // X prefetch distance in nonzeros (register window)
    int jit_nbuf = 1;                       // KLE value staging buffers per warp (1 or 2)
    int jit_diff_req = 1;                   // difference form asked for (SGFEM_JIT_DIFF)
    int jit_diff = 0;                       // difference form in use: FP32 apply as sum_j K_ij (x_j - x_i)
    bool rowsum_zero = false;               // every row of every K_m sums to zero (up to rounding)
    int jit_window_req = 1;                 // lattice-window kernel asked for (SGFEM_JIT_WINDOW)
    int jit_window = 0;                     // lattice-window kernel in use
    int jit_wwpb = 12;                      // its warps per block
    int jit_wrw = 2;                        // its rows per warp and lattice line
    int jit_unroll = 1;                     // its unroll of the nonzero loop (SGFEM_JIT_UNROLL)
    int jit_minb = 0;                       // minimum resident blocks per SM asked of ptxas (0: none)
    int jit_async = 0;                      // cp.async ring variant of the kernel
    int jit_adepth = 6;                     // ring slots (nonzeros in flight + 1) per warp
    int jit_stage = 1;                      // KLE values staged in shared memory
    int jit_bps_cap = 8;                    // resident blocks per SM used by the grid
    int jit_carveout = -1;                  // preferred shared-memory carve-out (%), -1 default
    void* jit_module = nullptr;             // CUmodule
    void* jit_func = nullptr;               // CUfunction
    int* d_jit_err = nullptr;               // status word of the specialised kernel
    bool jit_ok = false;
    bool jit_tried = false;      // the specialised FP32 apply is compiled at its first use
    bool jit_disabled = false;   // SGFEM_APPLY=generic at finalize
    int jit_blocks_per_sm = 1;
    std::string jit_log;

    // lattice preconditioner
    bool lattice = false;
    int Nl = 0;                 // lattice intervals per side; points (Nl+1)^2
    bool lat_order = false;     // device rows are the lattice points, row = y * lat_np + x
    int lat_np = 0;             // lattice points per line (Nl + 1)
    int win_hx = 0, win_hy = 0; // largest |dx|, |dy| between an interior row and its columns
    int lat_log2 = 0;           // Nl = 2^lat_log2
    double lat_scale = 1.0;     // a0: K_0 ~ a0 * L on interior rows
    double* d_lat_tab64 = nullptr;  // see lattice.cu
    float* d_lat_tab32 = nullptr;
    double* d_lat_scale64 = nullptr;  // per (kx, ky) scale, (Nl-1)^2
    float* d_lat_scale32 = nullptr;
    bool lat_block = false;         // exact K_0^-1 by 4x4 blocks of the sine transform (pass Y)
    double* d_lat_blk64 = nullptr;  // per (kx, ky) in [1, Nl/2]^2: 10 values of a symmetric 4x4 block
    float* d_lat_blk32 = nullptr;
    std::string lat_log;            // which mean-based preconditioner is in use, and why
    MeanChol* chol = nullptr;       // exact K_0^-1 on any mesh (factored at the first use)
    SmallPCG* small = nullptr;      // one-cluster inner PCG of the mixed solve (small lattice problems)

    // workspaces (lazily sized)
    DeviceBuf w_stage;         // host-layout staging (n*P doubles)
    DeviceBuf w_vec[SG_NBUF];  // SG vectors
    DeviceBuf w_partials;      // per-block reduction partials (double)
    DeviceBuf w_basis;         // GMRES Krylov basis (restart + 1 vectors)
    DeviceBuf w_zbasis;        // flexible GMRES: preconditioned basis vectors (restart, FP32)
    // PCG graph (a device loop of check_every iterations per body), kept for the next
    // run on the same buffers
    cudaGraph_t pcg_graph = nullptr;
    cudaGraphExec_t pcg_exec = nullptr;
    uint64_t pcg_key[13] = {};
    long long pcg_per_graph = 0;  // kernel launches per loop body
    DeviceBuf w_gsmall;        // GMRES multi-dot partials and coefficients
    KrylovScalars* d_scal = nullptr;
    KrylovScalars* h_scal = nullptr;  // pinned
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    // sgfem_solve into pinned host memory: the solution of a refinement step expected
    // to end the solve goes to the host on a side stream while the convergence check
    // (the FP64 / double-FP32 residual) runs
    cudaStream_t side = nullptr;
    cudaEvent_t ev_spec_x = nullptr, ev_spec = nullptr;  // x converted; copy done
    double* spec_host = nullptr;  // destination while a solve runs, else null
    bool spec_pending = false;    // a copy was issued (ev_spec marks its end)
    bool spec_valid = false;      // the last copy holds the current solution
    long long launches = 0;    // kernels launched by this context (graph replays included)
};

// ------------------------------------------------------------------ errors / memory
int sg_fail(sgfem_context* ctx, int code, const std::string& msg);
int sg_cuda_fail(sgfem_context* ctx, cudaError_t e, const char* what);

#define SG_CUDA(ctx, call)                                              \
    do {                                                                \
        cudaError_t _e = (call);                                        \
        if (_e != cudaSuccess) return sg_cuda_fail((ctx), _e, #call);   \
    } while (0)

// after a kernel launch: count it and check the launch
#define SG_LAUNCHED(ctx)                                   \
    do {                                                   \
        (ctx)->launches++;                                 \
        SG_CUDA(ctx, cudaGetLastError());                  \
    } while (0)

#define SG_TRY(call)                   \
    do {                               \
        int _s = (call);               \
        if (_s != SGFEM_OK) return _s; \
    } while (0)

int sg_ensure(sgfem_context* ctx, DeviceBuf& b, size_t bytes);
size_t sg_elem_bytes(int precision);
size_t sg_vec_bytes(const sgfem_context* ctx, int precision);
int sg_check_ready(sgfem_context* ctx);

// ------------------------------------------------------------------ apply (apply.cu)
// Y = S X in device layout.  If dot_partials != nullptr each block writes the FP64
// partial sum of X .* Y to dot_partials[block]; *nblocks receives the block count.
int sg_launch_apply(sgfem_context* ctx, int precision, const void* X, void* Y,
                    double* dot_partials, int* nblocks, const KrylovScalars* skip_if_done);

// ------------------------------------------------------------------ specialised apply (jit.cu)
void sg_mode_order(const sgfem_context* ctx, const std::vector<std::vector<char>>& nzcol,
                   std::vector<int32_t>& mode_of_col);
// compile the FP32 apply for this coupling structure; returns SGFEM_OK or an error
// (the generic kernel stays in use then)
void sg_jit_configure(sgfem_context* ctx);
int sg_jit_build(sgfem_context* ctx);
// compile it once, before the first FP32 apply of a context (never inside a graph capture)
int sg_jit_ensure(sgfem_context* ctx);
int sg_jit_grid(const sgfem_context* ctx);
int sg_jit_launch(sgfem_context* ctx, const void* X, void* Y, double* partials, int grid, const KrylovScalars* scal);
void sg_jit_release(sgfem_context* ctx);
// error status of the specialised kernel since the last check (resets it)
int sg_jit_check(sgfem_context* ctx);
// double-FP32 refinement residual (residual_df.cu): usable when every K_m has vanishing
// row sums (difference form); xs/bs are (hi, lo) float2 vectors in the device layout
bool sg_residual_df_usable(const sgfem_context* ctx);
int sg_residual_df_prepare(sgfem_context* ctx);
int sg_split_df(sgfem_context* ctx, double* x, const double* d, void* xs, int add);
int sg_residual_df(sgfem_context* ctx, const void* xs, const void* bs, float* r32, double* partials, int* nblocks);
// split-slot form of the lattice-window FP32 apply (jit_split.cu): plan and tables at the
// first FP32 use (needs the lattice window); source for NVRTC; shared memory; release
int sg_split_plan(sgfem_context* ctx, std::string& why);  // host only
int sg_split_upload(sgfem_context* ctx);
std::string sg_split_source(const sgfem_context* ctx);
size_t sg_split_smem(const sgfem_context* ctx, int wpb);
const int* sg_split_lanetab(const sgfem_context* ctx);
const int2* sg_split_jtab(const sgfem_context* ctx);
std::string sg_split_summary(const sgfem_context* ctx);
void sg_split_release(sgfem_context* ctx);
// whether the specialised kernel takes this X (the window kernel copies 16-byte pieces)
bool sg_jit_accepts(const sgfem_context* ctx, const void* X);

// ------------------------------------------------------------------ layout (context.cu)
int sg_launch_to_device(sgfem_context* ctx, const double* stage, void* X, int precision);
int sg_launch_from_device(sgfem_context* ctx, const void* X, double* stage, int precision);

// ------------------------------------------------------------------ preconditioners (lattice.cu)
int sg_lattice_setup(sgfem_context* ctx);
// largest block count of a lattice pass (size of the reduction partials)
int sg_lat_max_blocks(const sgfem_context* ctx);
// K(y_s) of every sample of a samples context into d_kval64/32 (after the values and
// the samples are on the device); leaves them null above a 4 GB budget
int sg_samples_combine(sgfem_context* ctx);
// exact mean preconditioner: K_0 restricted to interior lattice points is translation invariant
// per parity class (x % 2, y % 2); rowptr/col in device numbering, val64 (nnz x M1, K_0 at m = 0)
int sg_lattice_blocks(sgfem_context* ctx, const std::vector<int64_t>& rowptr, const std::vector<int32_t>& col,
                      const std::vector<double>& val64);
// pass 1: T = DST_x(R) on interior rows
int sg_lat_pass_x(sgfem_context* ctx, int precision, const void* R, void* T,
                  const KrylovScalars* skip_if_done);
// pass 2: T <- DST_y(scale .* DST_y(T)); rz partials (Parseval) if rz != nullptr
int sg_lat_pass_y(sgfem_context* ctx, int precision, void* T, double* rz, int* nblocks,
                  const KrylovScalars* skip_if_done);
// pass 3: z = DST_x(T); mode 0: out = z (boundary rows untouched), mode 1: out = z + beta*out
int sg_lat_pass_xinv(sgfem_context* ctx, int precision, const void* T, void* out, int mode,
                     const KrylovScalars* scal);
// Jacobi (identity=1: plain identity on interior rows): mode 0: out = D^-1 R ;
// mode 1: out = D^-1 R + beta*out on interior rows ; mode 2: r'z partials only
int sg_jacobi(sgfem_context* ctx, int precision, const void* R, void* out, int mode, int identity,
              double* rz, int* nblocks, const KrylovScalars* scal);
// mean-based preconditioner on any mesh by sparse Cholesky (meanchol.cu): K_0 of the
// interior rows is kept at finalize, factored at the first use (never inside a capture)
int sg_chol_prepare(sgfem_context* ctx, const std::vector<int64_t>& rowptr, const std::vector<int32_t>& col,
                    const std::vector<double>& val64);
int sg_chol_ensure(sgfem_context* ctx);
int sg_chol_workspace(sgfem_context* ctx, int precision);
// Z = K_0^-1 R on interior rows, boundary rows of Z zero
int sg_chol_apply(sgfem_context* ctx, int precision, const void* R, void* Z, const KrylovScalars* scal);
// mode 2: r'z partials; mode 1: P = Z + beta P (interior rows)
int sg_chol_finish(sgfem_context* ctx, int precision, const void* R, const void* Z, void* P, int mode, double* rz,
                   int* nblocks, const KrylovScalars* scal);
const char* sg_chol_log(const sgfem_context* ctx);
// one-cluster FP32 inner PCG (small.cu): eligibility and tables at finalize, coupling
// tables at the first use (again after a coupling update)
int sg_small_prepare(sgfem_context* ctx, const std::vector<int64_t>& rowptr, const std::vector<int32_t>& col,
                     const std::vector<double>& val64);
bool sg_small_usable(sgfem_context* ctx);
int sg_small_pcg_launch(sgfem_context* ctx, const float* r32, double* d64, int maxit);
void sg_small_pcg_result(const sgfem_context* ctx, int* iters, int* status);  // after a stream synchronisation
const char* sg_small_log(const sgfem_context* ctx);
void sg_small_invalidate(sgfem_context* ctx);
void sg_small_release(sgfem_context* ctx);
void sg_chol_release(sgfem_context* ctx);
// set the dynamic shared-memory limits once (before any graph capture)
int sg_lattice_configure(sgfem_context* ctx);
int sg_apply_configure(sgfem_context* ctx);
