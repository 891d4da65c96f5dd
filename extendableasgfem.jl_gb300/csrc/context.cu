// Context, operator setup and the host <-> device layout boundary of libsgfem.
//
// Replaces the construction side of the reference solver:
//   MySystemPrimal(A0, Am, G, bdofs, nmodes)   src/modelproblems/solvers_poisson_primal.jl:14-21,144
//   boundary dofs from FES[BFaceDofs]          solvers_poisson_primal.jl:136-142
// and the SGFEVector layout (src/sgfevector.jl:86-106): a caller vector is
// column-major n x P; on the device it becomes row-major n x ld (see
// sgfem_internal.h).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <numeric>

#include "sgfem_internal.h"

int sg_fail(sgfem_context* ctx, int code, const std::string& msg) {
    if (ctx) ctx->err = msg;
    return code;
}

int sg_cuda_fail(sgfem_context* ctx, cudaError_t e, const char* what) {
    std::string m = std::string("CUDA error in ") + what + ": " + cudaGetErrorString(e);
    return sg_fail(ctx, SGFEM_ERR_CUDA, m);
}

int sg_ensure(sgfem_context* ctx, DeviceBuf& b, size_t bytes) {
    if (b.bytes >= bytes && b.p) return SGFEM_OK;
    if (b.p) {
        SG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        SG_CUDA(ctx, cudaFree(b.p));
        b.p = nullptr;
        b.bytes = 0;
    }
    SG_CUDA(ctx, cudaMalloc(&b.p, bytes));
    b.bytes = bytes;
    return SGFEM_OK;
}

size_t sg_elem_bytes(int precision) { return precision == SGFEM_FP64 ? 8 : 4; }

size_t sg_vec_bytes(const sgfem_context* ctx, int precision) {
    return (size_t)ctx->n * (size_t)ctx->ld * sg_elem_bytes(precision);
}

int sg_check_ready(sgfem_context* ctx) {
    if (!ctx) return SGFEM_ERR_ARGUMENT;
    if (!ctx->finalized) return sg_fail(ctx, SGFEM_ERR_STATE, "sgfem_finalize has not been called");
    return SGFEM_OK;
}

static void free_dev(void* p) {
    if (p) cudaFree(p);
}

extern "C" int sgfem_version(void) { return 10000; }

extern "C" long long sgfem_kernel_launches(const sgfem_context* ctx) { return ctx ? ctx->launches : 0; }

extern "C" int sgfem_create(sgfem_context** out, int device) {
    if (!out) return SGFEM_ERR_ARGUMENT;
    *out = nullptr;
    sgfem_context* ctx = new sgfem_context();
    ctx->device = device;
    cudaError_t e = cudaSetDevice(device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, device);
    if (e == cudaSuccess) e = cudaMalloc(&ctx->d_scal, sizeof(KrylovScalars));
    if (e == cudaSuccess) e = cudaMallocHost(&ctx->h_scal, sizeof(KrylovScalars));
    if (e == cudaSuccess) e = cudaEventCreate(&ctx->ev0);
    if (e == cudaSuccess) e = cudaEventCreate(&ctx->ev1);
    if (e != cudaSuccess) {
        // report through a transient context so the caller sees the reason
        *out = ctx;
        return sg_cuda_fail(ctx, e, "sgfem_create");
    }
    *out = ctx;
    return SGFEM_OK;
}

extern "C" int sgfem_destroy(sgfem_context* ctx) {
    if (!ctx) return SGFEM_OK;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    void* ptrs[] = {ctx->d_rowptr, ctx->d_col, ctx->d_val64, ctx->d_val32, ctx->d_bmask, ctx->d_iperm,
                    ctx->d_dinv64, ctx->d_dinv32, ctx->d_qtab, ctx->d_combptr, ctx->d_combq,
                    ctx->d_combg64, ctx->d_combg32, ctx->d_lat_tab64, ctx->d_lat_tab32,
                    ctx->d_lat_scale64, ctx->d_lat_scale32, ctx->d_lat_blk64, ctx->d_lat_blk32, ctx->d_scal, ctx->w_stage.p, ctx->w_partials.p,
                    ctx->d_jptr, ctx->d_joff, ctx->d_jg, ctx->d_jtab, ctx->d_val32p, ctx->d_mode_of_col,
                    ctx->d_y64, ctx->d_y32, ctx->d_valdf, ctx->d_combgdf, ctx->d_kval64, ctx->d_kval32};
    if (ctx->pcg_exec) cudaGraphExecDestroy(ctx->pcg_exec);
    if (ctx->pcg_graph) cudaGraphDestroy(ctx->pcg_graph);
    sg_jit_release(ctx);
    sg_chol_release(ctx);
    sg_small_release(ctx);
    for (void* p : ptrs) free_dev(p);
    for (int i = 0; i < SG_NBUF; ++i) free_dev(ctx->w_vec[i].p);
    free_dev(ctx->w_basis.p);
    free_dev(ctx->w_zbasis.p);
    free_dev(ctx->w_gsmall.p);
    free_dev(ctx->w_valhl.p);
    free_dev(ctx->w_yhl.p);
    free_dev(ctx->w_samp.p);
    if (ctx->h_scal) cudaFreeHost(ctx->h_scal);
    if (ctx->ev0) cudaEventDestroy(ctx->ev0);
    if (ctx->ev1) cudaEventDestroy(ctx->ev1);
    if (ctx->side) cudaStreamSynchronize(ctx->side);
    if (ctx->ev_spec_x) cudaEventDestroy(ctx->ev_spec_x);
    if (ctx->ev_spec) cudaEventDestroy(ctx->ev_spec);
    if (ctx->side) cudaStreamDestroy(ctx->side);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
    return SGFEM_OK;
}

extern "C" const char* sgfem_last_error(const sgfem_context* ctx) {
    if (!ctx) return "null context";
    return ctx->err.c_str();
}

// ------------------------------------------------------------------ setup
static int invalidate(sgfem_context* ctx) {
    if (ctx->finalized) return sg_fail(ctx, SGFEM_ERR_STATE, "context already finalized");
    return SGFEM_OK;
}

extern "C" int sgfem_set_spatial_matrix(sgfem_context* ctx, int m, int64_t n, const int64_t* colptr,
                                        const int64_t* rowval, const double* nzval) {
    if (!ctx) return SGFEM_ERR_ARGUMENT;
    SG_TRY(invalidate(ctx));
    if (m < 0 || m > 4096 || n <= 0 || n > (int64_t)INT32_MAX || !colptr || !rowval || !nzval)
        return sg_fail(ctx, SGFEM_ERR_ARGUMENT, "sgfem_set_spatial_matrix: bad arguments");
    if (ctx->n >= 0 && ctx->n != n) return sg_fail(ctx, SGFEM_ERR_ARGUMENT, "matrix size differs from earlier matrices");
    int64_t nnz = colptr[n] - 1;
    if (colptr[0] != 1 || nnz < 0) return sg_fail(ctx, SGFEM_ERR_ARGUMENT, "colptr must be 1-based");
    HostCSC c;
    c.n = n;
    c.colptr.resize(n + 1);
    for (int64_t j = 0; j <= n; ++j) {
        c.colptr[j] = colptr[j] - 1;
        if (j > 0 && c.colptr[j] < c.colptr[j - 1]) return sg_fail(ctx, SGFEM_ERR_ARGUMENT, "colptr not monotone");
    }
    c.rowval.resize(nnz);
    c.nzval.assign(nzval, nzval + nnz);
    for (int64_t k = 0; k < nnz; ++k) {
        int64_t r = rowval[k] - 1;
        if (r < 0 || r >= n) return sg_fail(ctx, SGFEM_ERR_ARGUMENT, "rowval out of range");
        c.rowval[k] = r;
    }
    c.set = true;
    ctx->n = n;
    if ((int64_t)ctx->mats.size() <= m) ctx->mats.resize(m + 1);
    ctx->mats[m] = std::move(c);
    return SGFEM_OK;
}

static int parse_coupling(sgfem_context* ctx, int64_t P, int64_t M, const int64_t* colptr, const int64_t* rowval,
                          const double* nzval) {
    if (P <= 0 || P > 32767 || M < 0 || M > 4095 || !colptr || (!rowval && colptr[P] > 1))
        return sg_fail(ctx, SGFEM_ERR_ARGUMENT, "sgfem_set_coupling: bad sizes (P <= 32767, M <= 4095)");
    int64_t nnz = colptr[P] - 1;
    if (colptr[0] != 1 || nnz < 0) return sg_fail(ctx, SGFEM_ERR_ARGUMENT, "G colptr must be 1-based");
    ctx->G_colptr.assign(colptr, colptr + P + 1);
    for (auto& v : ctx->G_colptr) v -= 1;
    ctx->G_rowval.resize(nnz);
    for (int64_t k = 0; k < nnz; ++k) {
        int64_t r = rowval[k] - 1;
        if (r < 0 || r >= M * P) return sg_fail(ctx, SGFEM_ERR_ARGUMENT, "G rowval out of range");
        ctx->G_rowval[k] = r;
    }
    ctx->G_val.assign(nzval, nzval + nnz);
    ctx->P = P;
    ctx->M = M;
    ctx->has_G = true;
    return SGFEM_OK;
}

extern "C" int sgfem_set_coupling(sgfem_context* ctx, int64_t P, int64_t M, const int64_t* colptr,
                                  const int64_t* rowval, const double* nzval) {
    if (!ctx) return SGFEM_ERR_ARGUMENT;
    SG_TRY(invalidate(ctx));
    return parse_coupling(ctx, P, M, colptr, rowval, nzval);
}

static int upload_samples(sgfem_context* ctx);

extern "C" int sgfem_set_samples(sgfem_context* ctx, int64_t S, int64_t M, const double* y) {
    if (!ctx) return SGFEM_ERR_ARGUMENT;
    if (S <= 0 || S > 32767 || M < 0 || M > 4095 || (M > 0 && !y))
        return sg_fail(ctx, SGFEM_ERR_ARGUMENT, "sgfem_set_samples: bad sizes (S <= 32767, M <= 4095)");
    for (int64_t t = 0; t < M * S; ++t)
        if (!std::isfinite(y[t])) return sg_fail(ctx, SGFEM_ERR_NONFINITE, "non-finite sample");
    if (ctx->finalized) {
        // next batch of the same shape
        if (!ctx->batched || S != ctx->P || M != ctx->M)
            return sg_fail(ctx, SGFEM_ERR_STATE, "finalized context: new samples need the same S and M of a samples context");
        ctx->ysamp.assign(y, y + M * S);
        SG_CUDA(ctx, cudaSetDevice(ctx->device));
        return upload_samples(ctx);
    }
    ctx->ysamp.assign(y, y + M * S);
    ctx->P = S;
    ctx->M = M;
    ctx->batched = true;
    ctx->has_G = true;
    return SGFEM_OK;
}

extern "C" int sgfem_set_boundary_dofs(sgfem_context* ctx, int64_t count, const int64_t* bdofs) {
    if (!ctx) return SGFEM_ERR_ARGUMENT;
    SG_TRY(invalidate(ctx));
    if (count < 0 || (count > 0 && !bdofs)) return sg_fail(ctx, SGFEM_ERR_ARGUMENT, "bad boundary dof list");
    ctx->bdofs.resize(count);
    for (int64_t k = 0; k < count; ++k) ctx->bdofs[k] = bdofs[k] - 1;
    ctx->has_bdofs = true;
    return SGFEM_OK;
}

extern "C" int sgfem_set_dof_coordinates(sgfem_context* ctx, int64_t n, const double* xy) {
    if (!ctx) return SGFEM_ERR_ARGUMENT;
    SG_TRY(invalidate(ctx));
    if (n <= 0 || !xy) return sg_fail(ctx, SGFEM_ERR_ARGUMENT, "bad coordinates");
    ctx->dof_xy.assign(xy, xy + 2 * n);
    return SGFEM_OK;
}

extern "C" int sgfem_has_lattice(const sgfem_context* ctx) { return (ctx && ctx->lattice) ? 1 : 0; }
extern "C" const char* sgfem_lattice_log(const sgfem_context* ctx) {
    if (!ctx) return "";
    return ctx->lattice ? ctx->lat_log.c_str() : "no lattice preconditioner";
}

// lattice detection: every dof at (ix/Nl, iy/Nl), all (Nl+1)^2 points present once
static bool detect_lattice(sgfem_context* ctx, std::vector<int32_t>& iperm) {
    int64_t n = ctx->n;
    if ((int64_t)ctx->dof_xy.size() != 2 * n) return false;
    int64_t side = (int64_t)std::llround(std::sqrt((double)n));
    if (side * side != n || side < 3) return false;
    int Nl = (int)(side - 1);
    iperm.assign(n, -1);
    std::vector<char> seen(n, 0);
    for (int64_t i = 0; i < n; ++i) {
        double x = ctx->dof_xy[2 * i] * Nl, y = ctx->dof_xy[2 * i + 1] * Nl;
        double rx = std::nearbyint(x), ry = std::nearbyint(y);
        if (std::fabs(x - rx) > 1e-6 || std::fabs(y - ry) > 1e-6) return false;
        if (rx < 0 || ry < 0 || rx > Nl || ry > Nl) return false;
        int64_t r = (int64_t)ry * (Nl + 1) + (int64_t)rx;
        if (seen[r]) return false;
        seen[r] = 1;
        iperm[i] = (int32_t)r;
    }
    ctx->Nl = Nl;
    ctx->lat_np = Nl + 1;
    return true;
}

// Device column order of the P modes.  Column c belongs to group c/32 (one
// lane per column in the specialised apply).  For every pair p >= 1 of KLE
// terms (K_2p, K_2p+1) the apply spends one packed FMA per group that holds a
// column coupled to that pair (pair 0 holds K_0, which couples every column),
// so the order minimises
//   cost = sum_{p>=1} #{groups holding a column coupled to pair p}.
// Start: columns sorted by the number of pairs they couple to (hubs first);
// then simulated annealing over swaps of two columns in different groups
// (fixed seeds, incremental cost), best of four runs.
void sg_mode_order(const sgfem_context* ctx, const std::vector<std::vector<char>>& nzcol,
                   std::vector<int32_t>& mode_of_col) {
    const int64_t P = ctx->P, M = ctx->M;
    const int NP = (int)((M + 2) / 2);  // pairs 0..NP-1, pair 0 = (K_0, K_1)
    const int KG = (int)((P + 31) / 32);
    std::vector<std::vector<char>> part(P, std::vector<char>(NP, 0));
    std::vector<int> deg(P, 0);
    for (int64_t nu = 0; nu < P; ++nu)
        for (int pr = 1; pr < NP; ++pr) {
            for (int m = 2 * pr; m <= std::min<int64_t>(M, 2 * pr + 1); ++m)
                if (nzcol[m][nu]) part[nu][pr] = 1;
            deg[nu] += part[nu][pr];
        }
    std::vector<int32_t> start(P);
    std::iota(start.begin(), start.end(), 0);
    std::stable_sort(start.begin(), start.end(), [&](int a, int b) { return deg[a] > deg[b]; });
    mode_of_col = start;
    if (KG <= 1 || NP <= 1) return;

    auto delta_of = [&](const std::vector<int>& cnt, int n1, int n2, int a, int b) {
        int delta = 0;
        for (int pr = 1; pr < NP; ++pr) {
            const int d = part[n1][pr] - part[n2][pr];  // +1: a column of pair pr moves from a to b
            if (d == 0) continue;
            const int ca = cnt[(size_t)pr * KG + a], cb = cnt[(size_t)pr * KG + b];
            delta += ((ca - d) > 0) - (ca > 0) + ((cb + d) > 0) - (cb > 0);
        }
        return delta;
    };
    int best_cost = -1;
    const int iters = (int)std::min<int64_t>(400000, 2000 * P);
    for (int run = 0; run < 4; ++run) {
        std::vector<int32_t> order = start;
        std::vector<int> cnt((size_t)NP * KG, 0);
        for (int64_t c = 0; c < P; ++c)
            for (int pr = 1; pr < NP; ++pr) cnt[(size_t)pr * KG + c / 32] += part[order[c]][pr];
        int cost = 0;
        for (size_t t = 0; t < cnt.size(); ++t) cost += cnt[t] > 0;
        std::vector<int32_t> best_order = order;
        int run_best = cost;
        uint64_t rs = 0x9E3779B97F4A7C15ull * (uint64_t)(run + 1);
        auto rnd = [&]() {
            rs ^= rs << 13; rs ^= rs >> 7; rs ^= rs << 17;
            return rs;
        };
        for (int it = 0; it < iters; ++it) {
            const int64_t c1 = (int64_t)(rnd() % (uint64_t)P), c2 = (int64_t)(rnd() % (uint64_t)P);
            const int a = (int)(c1 / 32), b = (int)(c2 / 32);
            if (a == b) continue;
            const int n1 = order[c1], n2 = order[c2];
            const int delta = delta_of(cnt, n1, n2, a, b);
            const double T = 2.0 * (1.0 - (double)it / iters) + 1e-3;
            const double u = (double)(rnd() >> 11) * (1.0 / 9007199254740992.0);
            if (delta <= 0 || u < std::exp(-delta / T)) {
                for (int pr = 1; pr < NP; ++pr) {
                    const int d = part[n1][pr] - part[n2][pr];
                    cnt[(size_t)pr * KG + a] -= d;
                    cnt[(size_t)pr * KG + b] += d;
                }
                std::swap(order[c1], order[c2]);
                cost += delta;
                if (cost < run_best) {
                    run_best = cost;
                    best_order = order;
                }
            }
        }
        if (best_cost < 0 || run_best < best_cost) {
            best_cost = run_best;
            mode_of_col = best_order;
        }
    }
}

template <typename T>
static int upload(sgfem_context* ctx, T** dst, const T* src, size_t count) {
    SG_CUDA(ctx, cudaMalloc((void**)dst, std::max<size_t>(count, 1) * sizeof(T)));
    if (count) SG_CUDA(ctx, cudaMemcpy(*dst, src, count * sizeof(T), cudaMemcpyHostToDevice));
    return SGFEM_OK;
}

// per-sample coefficient rows [S][M1], y_{s,0} = 1, to d_y64 / d_y32 (allocated on first use)
static int upload_samples(sgfem_context* ctx) {
    const int64_t S = ctx->P, M = ctx->M, M1 = M + 1;
    std::vector<double> y64((size_t)S * M1);
    std::vector<float> y32((size_t)S * M1);
    for (int64_t sidx = 0; sidx < S; ++sidx) {
        y64[(size_t)sidx * M1] = 1.0;
        for (int64_t m = 1; m <= M; ++m) y64[(size_t)sidx * M1 + m] = ctx->ysamp[(size_t)sidx * M + (m - 1)];
    }
    for (size_t t = 0; t < y64.size(); ++t) y32[t] = (float)y64[t];
    if (!ctx->d_y64) {
        SG_TRY(upload(ctx, &ctx->d_y64, y64.data(), y64.size()));
        SG_TRY(upload(ctx, &ctx->d_y32, y32.data(), y32.size()));
    } else {
        SG_CUDA(ctx, cudaMemcpy(ctx->d_y64, y64.data(), y64.size() * sizeof(double), cudaMemcpyHostToDevice));
        SG_CUDA(ctx, cudaMemcpy(ctx->d_y32, y32.data(), y32.size() * sizeof(float), cudaMemcpyHostToDevice));
    }
    ctx->samples_x_valid = false;
    if (ctx->d_val64) SG_TRY(sg_samples_combine(ctx));  // next batch of a finalized context
    return SGFEM_OK;
}


// row stride of SG vectors in the device layout: P rounded up to `align` values
static void set_ld(sgfem_context* ctx) {
    const char* ea = getenv("SGFEM_LD_ALIGN");
    int align = ea ? atoi(ea) : 4;
    if (align != 4 && align != 8 && align != 16 && align != 32) align = 4;
    ctx->ld = (ctx->P + align - 1) / align * align;
}

// Coupling-dependent state of a finalized context (everything that depends on G
// and P): device column order, pair list and combination tables, slot tables
// and lane schedule of the specialised FP32 apply.  val64 (nnz x M1) is given at
// finalize to build the padded FP32 values; a coupling update passes nullptr and
// keeps them.
static int build_coupling(sgfem_context* ctx, const std::vector<double>* val64, int64_t nnz) {
        const int64_t M = ctx->M, P = ctx->P;
    // ---- coupling structure from G ((M*P) x P, CSC): entry (row = m'*P + mu, col = nu), m = m'+1
        std::vector<std::vector<char>> nzcol(M + 1, std::vector<char>(P, 0));
        struct GE { int m; int mu; int nu; double g; };
        std::vector<GE> ges;
        for (int64_t nu = 0; nu < P; ++nu)
            for (int64_t k = ctx->G_colptr[nu]; k < ctx->G_colptr[nu + 1]; ++k) {
                double g = ctx->G_val[k];
                if (g == 0.0) continue;  // the reference skips zero couplings (solvers_poisson_primal.jl:111)
                int64_t r = ctx->G_rowval[k];
                int m = (int)(r / P) + 1;
                int mu = (int)(r % P);
                nzcol[m][nu] = 1;
                ges.push_back({m, mu, (int)nu, g});
            }
    
        // ---- device column order of the modes (sg_mode_order): packs the coupled
        // columns of each pair of KLE terms into few 32-column groups
        std::vector<int32_t> mode_of_col;  // device column -> caller mode
        sg_mode_order(ctx, nzcol, mode_of_col);
        ctx->imode.assign(P, 0);
        for (int64_t c = 0; c < P; ++c) ctx->imode[mode_of_col[c]] = (int32_t)c;
        const std::vector<int32_t>& imode = ctx->imode;
    
        // pair list Q in device columns: (0, c) for all c, then (m, c) for nonzero columns of G_m
        std::vector<int32_t> qtab;
        std::map<std::pair<int, int>, int> qidx;
        for (int64_t c = 0; c < P; ++c) {
            qidx[{0, (int)c}] = (int)qtab.size();
            qtab.push_back((int32_t)c);
        }
        for (int64_t m = 1; m <= M; ++m)
            for (int64_t c = 0; c < P; ++c)
                if (nzcol[m][mode_of_col[c]]) {
                    qidx[{(int)m, (int)c}] = (int)qtab.size();
                    qtab.push_back((int32_t)((m << 16) | c));
                }
        ctx->Qn = (int)qtab.size();
        for (GE& e : ges) {
            e.mu = imode[e.mu];
            e.nu = imode[e.nu];
        }
        std::sort(ges.begin(), ges.end(), [](const GE& a, const GE& b) {
            if (a.mu != b.mu) return a.mu < b.mu;
            if (a.m != b.m) return a.m < b.m;
            return a.nu < b.nu;
        });
        std::vector<int32_t> combptr(P + 1, 0), combq;
        std::vector<double> combg;
        for (const GE& e : ges) {
            combptr[e.mu + 1]++;
            combq.push_back(qidx[{e.m, e.nu}]);
            combg.push_back(e.g);
        }
        for (int64_t mu = 0; mu < P; ++mu) combptr[mu + 1] += combptr[mu];
        ctx->ncomb = (int)combq.size();
        std::vector<float> combg32(combg.begin(), combg.end());
    
        // ---- slot tables of the specialised FP32 apply: slot (pair p = m/2, group k = c/32)
        // exists if some column of group k couples to K_2p or K_2p+1 (K_0 couples to all).
        // The column groups are split into jit_np passes (contiguous group ranges with
        // balanced slot counts); a pass keeps only its own slots' accumulators.  Slots are
        // numbered pass by pass; jit_pass_slot0[p] is the first slot of pass p.
        sg_jit_configure(ctx);
        const int KG = (int)((P + 31) / 32);
        const int NPAIR = (ctx->M1 + 1) / 2;
        ctx->M1P = (ctx->M1 + 3) / 4 * 4;
        std::vector<std::vector<char>> needs(NPAIR, std::vector<char>(KG, 0));
        std::vector<int> slots_in_group(KG, 0);
        for (int pr = 0; pr < NPAIR; ++pr)
            for (int k = 0; k < KG; ++k) {
                bool need = false;
                for (int c = 32 * k; c < std::min<int64_t>(P, 32 * k + 32) && !need; ++c)
                    for (int m = 2 * pr; m <= std::min<int64_t>(M, 2 * pr + 1) && !need; ++m)
                        need = (m == 0) || nzcol[m][mode_of_col[c]];
                needs[pr][k] = need;
                slots_in_group[k] += need;
            }
        const int np = std::max(1, std::min(ctx->jit_np_req, KG));
        ctx->jit_pass_k0.assign(np + 1, KG);
        {
            int total = 0;
            for (int k = 0; k < KG; ++k) total += slots_in_group[k];
            int p = 0, acc = 0;
            ctx->jit_pass_k0[0] = 0;
            for (int k = 0; k < KG; ++k) {
                // close pass p once it holds its share and groups remain for the others
                if (p + 1 < np && acc > 0 && acc + slots_in_group[k] / 2 > (long long)total * (p + 1) / np &&
                    KG - k >= np - p - 1) {
                    ctx->jit_pass_k0[++p] = k;
                }
                acc += slots_in_group[k];
            }
            for (int q = p + 1; q <= np; ++q) ctx->jit_pass_k0[q] = KG;
            ctx->jit_np = p + 1;
            ctx->jit_pass_k0.resize(ctx->jit_np + 1);
            ctx->jit_pass_k0[ctx->jit_np] = KG;
        }
        std::vector<int> pass_of_k(KG, 0);
        for (int p = 0; p < ctx->jit_np; ++p)
            for (int k = ctx->jit_pass_k0[p]; k < ctx->jit_pass_k0[p + 1]; ++k) pass_of_k[k] = p;
        ctx->jit_slot_of.assign((size_t)NPAIR * KG, -1);
        ctx->jit_slots.clear();
        ctx->jit_pass_slot0.assign(ctx->jit_np + 1, 0);
        for (int p = 0; p < ctx->jit_np; ++p) {
            ctx->jit_pass_slot0[p] = (int)ctx->jit_slots.size();
            for (int pr = 0; pr < NPAIR; ++pr)
                for (int k = ctx->jit_pass_k0[p]; k < ctx->jit_pass_k0[p + 1]; ++k)
                    if (needs[pr][k]) {
                        ctx->jit_slot_of[(size_t)pr * KG + k] = (int)ctx->jit_slots.size();
                        ctx->jit_slots.push_back({pr, k});
                    }
        }
        ctx->jit_pass_slot0[ctx->jit_np] = (int)ctx->jit_slots.size();
        // sacc offset of F(m, c) within its pass's accumulator block
        auto slot_off = [&](int m, int c) {
            const int sl = ctx->jit_slot_of[(size_t)(m / 2) * KG + c / 32];
            const int ls = sl - ctx->jit_pass_slot0[pass_of_k[c / 32]];
            return ls * 64 + 2 * (c % 32) + (m % 2);
        };
        auto pass_of = [&](int c) { return pass_of_k[c / 32]; };
        // combination list per output column: (1, acc(0, c)) then (g, acc(m, nu)); jpass is
        // the pass whose accumulators hold the entry
        std::vector<int32_t> jptr(P + 1, 0), joff, jpass;
        std::vector<float> jg;
        for (int64_t c = 0; c < P; ++c) {
            joff.push_back(slot_off(0, (int)c));
            jpass.push_back(pass_of((int)c));
            jg.push_back(1.0f);
            for (int32_t e = combptr[c]; e < combptr[c + 1]; ++e) {
                int q = combq[e];
                int m = qtab[q] >> 16, nu = qtab[q] & 0xffff;
                joff.push_back(slot_off(m, nu));
                jpass.push_back(pass_of(nu));
                jg.push_back((float)combg[e]);
            }
            jptr[c + 1] = (int32_t)joff.size();
        }
        std::vector<float> val32p;
        if (val64) {  // the padded FP32 values depend on the K_m only: kept by a coupling update
            val32p.assign((size_t)nnz * ctx->M1P, 0.0f);
            for (int64_t k = 0; k < nnz; ++k)
                for (int m = 0; m < ctx->M1; ++m)
                    val32p[(size_t)k * ctx->M1P + m] = (float)(*val64)[(size_t)k * ctx->M1 + m];
        }
        SG_TRY(upload(ctx, &ctx->d_jptr, jptr.data(), jptr.size()));
        SG_TRY(upload(ctx, &ctx->d_joff, joff.data(), joff.size()));
        SG_TRY(upload(ctx, &ctx->d_jg, jg.data(), jg.size()));
        // lane schedule of the combination: columns assigned to the 32 lanes longest
        // first (each to the least loaded lane); per lane its columns' entries in
        // sequence, padded to a common length T; entry (i, lane) at [i * 32 + lane]
        // x = sacc offset | column << 13 | (last entry of the column) << 28, y = g bits
        {
            std::vector<int> order(P);
            std::iota(order.begin(), order.end(), 0);
            std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
                return (jptr[a + 1] - jptr[a]) > (jptr[b + 1] - jptr[b]);
            });
            const int NPS = ctx->jit_np;
            // lanes[p][l]: lane l's entries of pass p; a column stays on one lane in every pass
            std::vector<std::vector<std::vector<int2>>> lanes(NPS, std::vector<std::vector<int2>>(32));
            std::vector<size_t> load(32, 0);
            for (int c : order) {
                int best = 0;
                for (int l = 1; l < 32; ++l)
                    if (load[l] < load[best]) best = l;
                load[best] += jptr[c + 1] - jptr[c];
                for (int p = 0; p < NPS; ++p) {
                    int lastp = -1;
                    for (int32_t e = jptr[c]; e < jptr[c + 1]; ++e)
                        if (jpass[e] == p) lastp = e;
                    for (int32_t e = jptr[c]; e < jptr[c + 1]; ++e) {
                        if (jpass[e] != p) continue;
                        int bits;
                        std::memcpy(&bits, &jg[e], sizeof(int));
                        const bool last = (e == lastp);
                        lanes[p][best].push_back(make_int2(joff[e] | (int)(c << 13) | ((last ? 1 : 0) << 28), bits));
                    }
                }
            }
            ctx->jit_pass_T.assign(NPS, 0);
            size_t T = 0;
            for (int p = 0; p < NPS; ++p) {
                size_t tp = 0;
                for (auto& l : lanes[p]) tp = std::max(tp, l.size());
                ctx->jit_pass_T[p] = (int)tp;
                T += tp;
            }
            ctx->jit_T = (int)T;
            std::vector<int2> jtab(std::max<size_t>(T, 1) * 32, make_int2(0, 0));
            size_t off = 0;
            for (int p = 0; p < NPS; ++p) {
                for (int l = 0; l < 32; ++l)
                    for (size_t i = 0; i < lanes[p][l].size(); ++i) jtab[(off + i) * 32 + l] = lanes[p][l][i];
                off += ctx->jit_pass_T[p];
            }
            int maxps = 0;
            for (int p = 0; p < NPS; ++p) maxps = std::max(maxps, ctx->jit_pass_slot0[p + 1] - ctx->jit_pass_slot0[p]);
            const bool fits = ((size_t)maxps * 64 <= 8192) && P <= 32767;
            if (!fits) ctx->jit_T = -1;
            SG_TRY(upload(ctx, &ctx->d_jtab, jtab.data(), jtab.size()));
        }
        if (val64) SG_TRY(upload(ctx, &ctx->d_val32p, val32p.data(), val32p.size()));
        ctx->mode_of_col = mode_of_col;
        SG_TRY(upload(ctx, &ctx->d_mode_of_col, mode_of_col.data(), mode_of_col.size()));
        SG_TRY(upload(ctx, &ctx->d_qtab, qtab.data(), qtab.size()));
        SG_TRY(upload(ctx, &ctx->d_combptr, combptr.data(), combptr.size()));
        SG_TRY(upload(ctx, &ctx->d_combq, combq.data(), combq.size()));
        SG_TRY(upload(ctx, &ctx->d_combg64, combg.data(), combg.size()));
        SG_TRY(upload(ctx, &ctx->d_combg32, combg32.data(), combg32.size()));
        ctx->h_qtab = qtab;
        ctx->h_combptr = combptr;
        ctx->h_combq = combq;
        ctx->h_combg = combg;
    return SGFEM_OK;
}

extern "C" int sgfem_finalize(sgfem_context* ctx) {
    if (!ctx) return SGFEM_ERR_ARGUMENT;
    SG_TRY(invalidate(ctx));
    SG_CUDA(ctx, cudaSetDevice(ctx->device));
    if (!ctx->has_G) return sg_fail(ctx, SGFEM_ERR_STATE, "coupling matrix not set");
    if (!ctx->has_bdofs) return sg_fail(ctx, SGFEM_ERR_STATE, "boundary dofs not set");
    const int64_t M = ctx->M, P = ctx->P, n = ctx->n;
    if ((int64_t)ctx->mats.size() < M + 1) return sg_fail(ctx, SGFEM_ERR_STATE, "spatial matrices K_0..K_M not all set");
    for (int64_t m = 0; m <= M; ++m)
        if (!ctx->mats[m].set) return sg_fail(ctx, SGFEM_ERR_STATE, "spatial matrix K_" + std::to_string(m) + " not set");
    ctx->M1 = (int)(M + 1);
    set_ld(ctx);
    for (int64_t b : ctx->bdofs)
        if (b < 0 || b >= n) return sg_fail(ctx, SGFEM_ERR_ARGUMENT, "boundary dof out of range");

    // ---- numbering
    std::vector<int32_t> iperm;
    ctx->lattice = detect_lattice(ctx, iperm);
    ctx->lat_order = ctx->lattice;
    if (!ctx->lattice) {
        iperm.resize(n);
        std::iota(iperm.begin(), iperm.end(), 0);
    }
    ctx->iperm = iperm;
    ctx->perm.assign(n, 0);
    for (int64_t i = 0; i < n; ++i) ctx->perm[iperm[i]] = (int32_t)i;

    // ---- union pattern (CSR in device numbering); K_m are given as CSC in caller numbering
    bool same = true;
    for (int64_t m = 1; m <= M && same; ++m) {
        same = ctx->mats[m].colptr == ctx->mats[0].colptr && ctx->mats[m].rowval == ctx->mats[0].rowval;
    }
    // entries (devrow, devcol) of the union pattern
    std::vector<int64_t> rowcount(n + 1, 0);
    std::vector<std::vector<std::pair<int32_t, int64_t>>> rows;  // unused when same
    std::vector<int32_t> col;
    std::vector<int64_t> rowptr(n + 1, 0);
    if (same) {
        const HostCSC& A = ctx->mats[0];
        // CSC of A in caller numbering == CSR of A^T; row i of A = column entries with rowval == i
        for (int64_t j = 0; j < n; ++j)
            for (int64_t k = A.colptr[j]; k < A.colptr[j + 1]; ++k) rowcount[iperm[A.rowval[k]] + 1]++;
    } else {
        // merge: collect all (devrow, devcol) keys, dedupe
        std::vector<int64_t> keys;
        for (int64_t m = 0; m <= M; ++m) {
            const HostCSC& A = ctx->mats[m];
            for (int64_t j = 0; j < n; ++j)
                for (int64_t k = A.colptr[j]; k < A.colptr[j + 1]; ++k)
                    keys.push_back((int64_t)iperm[A.rowval[k]] * n + iperm[j]);
        }
        std::sort(keys.begin(), keys.end());
        keys.erase(std::unique(keys.begin(), keys.end()), keys.end());
        col.resize(keys.size());
        for (size_t t = 0; t < keys.size(); ++t) {
            rowcount[keys[t] / n + 1]++;
            col[t] = (int32_t)(keys[t] % n);
        }
    }
    for (int64_t i = 0; i < n; ++i) rowptr[i + 1] = rowptr[i] + rowcount[i + 1];
    const int64_t nnz = rowptr[n];
    ctx->row_nnz_max = 0;
    for (int64_t i = 0; i < n; ++i) ctx->row_nnz_max = std::max<int>(ctx->row_nnz_max, (int)rowcount[i + 1]);
    if (nnz > (int64_t)INT32_MAX) return sg_fail(ctx, SGFEM_ERR_UNSUPPORTED, "more than 2^31 nonzeros");
    ctx->nnz = nnz;
    if (same) {
        col.assign(nnz, 0);
        std::vector<int64_t> fill(rowptr.begin(), rowptr.end() - 1);
        const HostCSC& A = ctx->mats[0];
        for (int64_t j = 0; j < n; ++j)
            for (int64_t k = A.colptr[j]; k < A.colptr[j + 1]; ++k) col[fill[iperm[A.rowval[k]]]++] = iperm[j];
        for (int64_t i = 0; i < n; ++i) std::sort(col.begin() + rowptr[i], col.begin() + rowptr[i + 1]);
    }
    // values: locate each (row, col) by binary search in the row
    const int M1 = ctx->M1;
    std::vector<double> val64((size_t)nnz * M1, 0.0);
    for (int64_t m = 0; m <= M; ++m) {
        const HostCSC& A = ctx->mats[m];
        for (int64_t j = 0; j < n; ++j) {
            int32_t cj = iperm[j];
            for (int64_t k = A.colptr[j]; k < A.colptr[j + 1]; ++k) {
                int32_t r = iperm[A.rowval[k]];
                auto b = col.begin() + rowptr[r], e = col.begin() + rowptr[r + 1];
                auto it = std::lower_bound(b, e, cj);
                val64[(size_t)(it - col.begin()) * M1 + m] += A.nzval[k];
            }
        }
    }
    std::vector<float> val32(val64.size());
    for (size_t t = 0; t < val64.size(); ++t) val32[t] = (float)val64[t];
    std::vector<int32_t> rowptr32(n + 1);
    for (int64_t i = 0; i <= n; ++i) rowptr32[i] = (int32_t)rowptr[i];

    // boundary mask and Jacobi diagonal
    ctx->bmask_host.assign(n, 0);
    for (int64_t b : ctx->bdofs) ctx->bmask_host[iperm[b]] = 1;
    std::vector<double> dinv(n, 0.0);
    std::vector<float> dinv32(n, 0.0f);
    double dsum = 0.0;
    int64_t dcount = 0;
    for (int64_t i = 0; i < n; ++i) {
        double d = 0.0;
        for (int64_t k = rowptr[i]; k < rowptr[i + 1]; ++k)
            if (col[k] == i) d = val64[(size_t)k * M1 + 0];
        if (!ctx->bmask_host[i]) {
            if (!(d > 0.0)) return sg_fail(ctx, SGFEM_ERR_ARGUMENT, "K_0 has a non-positive interior diagonal entry");
            dinv[i] = 1.0 / d;
            dinv32[i] = (float)dinv[i];
            dsum += d;
            dcount++;
        }
    }
    ctx->lat_scale = dcount ? dsum / (4.0 * dcount) : 1.0;
    // lattice reach of the couplings (interior rows), for the window kernel
    ctx->win_hx = ctx->win_hy = 0;
    if (ctx->lat_order) {
        const int np = ctx->lat_np;
        for (int64_t i = 0; i < n; ++i) {
            if (ctx->bmask_host[i]) continue;
            const int iy = (int)(i / np), ix = (int)(i % np);
            for (int64_t k = rowptr[i]; k < rowptr[i + 1]; ++k) {
                const int jy = col[k] / np, jx = col[k] % np;
                ctx->win_hx = std::max(ctx->win_hx, std::abs(jx - ix));
                ctx->win_hy = std::max(ctx->win_hy, std::abs(jy - iy));
            }
        }
    }
    // vanishing row sums of every K_m on the interior rows (stiffness and convection
    // blocks without eliminated boundary columns) allow the difference-form FP32 apply
    ctx->rowsum_zero = true;
    for (int64_t i = 0; i < n && ctx->rowsum_zero; ++i) {
        if (ctx->bmask_host[i]) continue;
        for (int m = 0; m < M1; ++m) {
            double sum = 0.0, asum = 0.0;
            for (int64_t k = rowptr[i]; k < rowptr[i + 1]; ++k) {
                sum += val64[(size_t)k * M1 + m];
                asum += fabs(val64[(size_t)k * M1 + m]);
            }
            if (fabs(sum) > 1e-10 * asum) { ctx->rowsum_zero = false; break; }
        }
    }

    if (ctx->batched) {
        // block-diagonal sample operator: identity mode order, per-sample coefficients
        std::vector<int32_t> ident(P);
        std::iota(ident.begin(), ident.end(), 0);
        ctx->mode_of_col = ident;
        ctx->imode = ident;
        SG_TRY(upload(ctx, &ctx->d_mode_of_col, ident.data(), ident.size()));
        SG_TRY(upload_samples(ctx));
        ctx->Qn = 0;
    } else {
        SG_TRY(build_coupling(ctx, &val64, nnz));
    }

    // ---- upload
    SG_TRY(upload(ctx, &ctx->d_rowptr, rowptr32.data(), rowptr32.size()));
    SG_TRY(upload(ctx, &ctx->d_col, col.data(), col.size()));
    SG_TRY(upload(ctx, &ctx->d_val64, val64.data(), val64.size()));
    SG_TRY(upload(ctx, &ctx->d_val32, val32.data(), val32.size()));
    if (ctx->batched) SG_TRY(sg_samples_combine(ctx));
    SG_TRY(upload(ctx, &ctx->d_bmask, ctx->bmask_host.data(), ctx->bmask_host.size()));
    SG_TRY(upload(ctx, &ctx->d_iperm, ctx->iperm.data(), ctx->iperm.size()));
    SG_TRY(upload(ctx, &ctx->d_dinv64, dinv.data(), dinv.size()));
    SG_TRY(upload(ctx, &ctx->d_dinv32, dinv32.data(), dinv32.size()));

    if (ctx->lattice) {
        int s = sg_lattice_setup(ctx);
        if (s == SGFEM_OK) s = sg_lattice_blocks(ctx, rowptr, col, val64);
        if (s != SGFEM_OK) {
            if (s == SGFEM_ERR_UNSUPPORTED) {
                ctx->lattice = false;  // e.g. Nl not a power of two: Jacobi only
                ctx->err.clear();
            } else {
                return s;
            }
        }
    }
    // exact mean preconditioner for any mesh: K_0 of the interior rows kept, factored at the first use
    SG_TRY(sg_chol_prepare(ctx, rowptr, col, val64));
    // one-cluster inner PCG for small P1 lattice problems (mixed solves)
    if (!ctx->batched) SG_TRY(sg_small_prepare(ctx, rowptr, col, val64));
    if (!ctx->batched) SG_TRY(sg_apply_configure(ctx));
    if (ctx->lattice) SG_TRY(sg_lattice_configure(ctx));

    // specialised FP32 apply; on failure the generic kernel stays in use (reason in the variant log)
    ctx->jit_log = ctx->batched ? "block-diagonal sample operator" : "not compiled yet (at the first FP32 apply)";
    // host copies of the pattern are no longer needed
    for (auto& A : ctx->mats) {
        A.colptr.clear(); A.colptr.shrink_to_fit();
        A.rowval.clear(); A.rowval.shrink_to_fit();
        A.nzval.clear(); A.nzval.shrink_to_fit();
    }
    ctx->finalized = true;
    return SGFEM_OK;
}

// New modes (the adaptive loop appends multi-indices, scripts/poisson.jl:341-420,
// mopcontrol.jl:60-132) change G and P but not the K_m: rebuild only the
// coupling-dependent state of a finalized context.  M may not exceed the number
// of K_m the context holds.
extern "C" int sgfem_update_coupling(sgfem_context* ctx, int64_t P, int64_t M, const int64_t* colptr,
                                     const int64_t* rowval, const double* nzval) {
    if (!ctx) return SGFEM_ERR_ARGUMENT;
    if (!ctx->finalized || ctx->batched)
        return sg_fail(ctx, SGFEM_ERR_STATE, "sgfem_update_coupling: needs a finalized SG (not samples) context");
    if (M > ctx->M1 - 1)
        return sg_fail(ctx, SGFEM_ERR_STATE,
                       "sgfem_update_coupling: more KLE terms than the context holds (finalize a new context)");
    SG_CUDA(ctx, cudaSetDevice(ctx->device));
    SG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    SG_TRY(parse_coupling(ctx, P, M, colptr, rowval, nzval));
    void** tabs[] = {(void**)&ctx->d_mode_of_col, (void**)&ctx->d_qtab, (void**)&ctx->d_combptr,
                     (void**)&ctx->d_combq, (void**)&ctx->d_combg64, (void**)&ctx->d_combg32,
                     (void**)&ctx->d_jptr, (void**)&ctx->d_joff, (void**)&ctx->d_jg, (void**)&ctx->d_jtab,
                     (void**)&ctx->d_combgdf};
    for (void** t : tabs) {
        free_dev(*t);
        *t = nullptr;
    }
    sg_jit_release(ctx);
    sg_small_invalidate(ctx);
    ctx->jit_tried = false;
    if (ctx->pcg_exec) cudaGraphExecDestroy(ctx->pcg_exec);
    if (ctx->pcg_graph) cudaGraphDestroy(ctx->pcg_graph);
    ctx->pcg_exec = nullptr;
    ctx->pcg_graph = nullptr;
    ctx->samples_x_valid = false;
    set_ld(ctx);
    SG_TRY(build_coupling(ctx, nullptr, ctx->nnz));
    SG_TRY(sg_apply_configure(ctx));
    ctx->jit_log = "not compiled yet (at the first FP32 apply)";
    return SGFEM_OK;
}

// ------------------------------------------------------------------ layout kernels// ------------------------------------------------------------------ layout kernels
// stage: caller layout, FP64, column-major n x P.  X: device layout (T), n x ld.
// tile of 32 dofs x 32 device columns; column c holds caller mode mode_of_col[c]
// (pad columns c >= P are written as zero)
template <typename T>
__global__ void k_to_device(const double* __restrict__ stage, T* __restrict__ X, const int* __restrict__ iperm,
                            const int* __restrict__ mode_of_col, int n, int P, int ld) {
    __shared__ double tile[32][33];
    int i0 = blockIdx.x * 32, c0 = blockIdx.y * 32;
    int tx = threadIdx.x, ty = threadIdx.y;  // 32 x 8
    for (int r = ty; r < 32; r += 8) {
        int c = c0 + r, i = i0 + tx;
        tile[r][tx] = (c < P && i < n) ? stage[(size_t)mode_of_col[c] * n + i] : 0.0;
    }
    __syncthreads();
    for (int r = ty; r < 32; r += 8) {
        int i = i0 + r, c = c0 + tx;
        if (i < n && c < ld) X[(size_t)iperm[i] * ld + c] = (T)tile[tx][r];
    }
}

template <typename T>
__global__ void k_from_device(const T* __restrict__ X, double* __restrict__ stage, const int* __restrict__ iperm,
                              const int* __restrict__ mode_of_col, int n, int P, int ld) {
    __shared__ double tile[32][33];
    int i0 = blockIdx.x * 32, c0 = blockIdx.y * 32;
    int tx = threadIdx.x, ty = threadIdx.y;
    for (int r = ty; r < 32; r += 8) {
        int i = i0 + r, c = c0 + tx;
        tile[r][tx] = (i < n && c < P) ? (double)X[(size_t)iperm[i] * ld + c] : 0.0;
    }
    __syncthreads();
    for (int r = ty; r < 32; r += 8) {
        int c = c0 + r, i = i0 + tx;
        if (c < P && i < n) stage[(size_t)mode_of_col[c] * n + i] = tile[tx][r];
    }
}

int sg_launch_to_device(sgfem_context* ctx, const double* stage, void* X, int precision) {
    dim3 block(32, 8), grid((unsigned)((ctx->n + 31) / 32), (unsigned)((ctx->ld + 31) / 32));
    if (precision == SGFEM_FP64)
        k_to_device<double><<<grid, block, 0, ctx->stream>>>(stage, (double*)X, ctx->d_iperm, ctx->d_mode_of_col, (int)ctx->n, (int)ctx->P, (int)ctx->ld);
    else
        k_to_device<float><<<grid, block, 0, ctx->stream>>>(stage, (float*)X, ctx->d_iperm, ctx->d_mode_of_col, (int)ctx->n, (int)ctx->P, (int)ctx->ld);
    SG_LAUNCHED(ctx);
    return SGFEM_OK;
}

int sg_launch_from_device(sgfem_context* ctx, const void* X, double* stage, int precision) {
    dim3 block(32, 8), grid((unsigned)((ctx->n + 31) / 32), (unsigned)((ctx->P + 31) / 32));
    if (precision == SGFEM_FP64)
        k_from_device<double><<<grid, block, 0, ctx->stream>>>((const double*)X, stage, ctx->d_iperm, ctx->d_mode_of_col, (int)ctx->n, (int)ctx->P, (int)ctx->ld);
    else
        k_from_device<float><<<grid, block, 0, ctx->stream>>>((const float*)X, stage, ctx->d_iperm, ctx->d_mode_of_col, (int)ctx->n, (int)ctx->P, (int)ctx->ld);
    SG_LAUNCHED(ctx);
    return SGFEM_OK;
}

static int check_precision(sgfem_context* ctx, int precision) {
    if (precision != SGFEM_FP64 && precision != SGFEM_FP32)
        return sg_fail(ctx, SGFEM_ERR_ARGUMENT, "precision must be SGFEM_FP64 or SGFEM_FP32");
    return SGFEM_OK;
}

// host vector (caller layout) -> device buffer (device layout)
static int host_to_device_layout(sgfem_context* ctx, const double* x, void* dst, int precision) {
    size_t hb = (size_t)ctx->n * ctx->P * sizeof(double);
    SG_TRY(sg_ensure(ctx, ctx->w_stage, hb));
    SG_CUDA(ctx, cudaMemcpyAsync(ctx->w_stage.p, x, hb, cudaMemcpyHostToDevice, ctx->stream));
    return sg_launch_to_device(ctx, (const double*)ctx->w_stage.p, dst, precision);
}

static int device_to_host_layout(sgfem_context* ctx, const void* src, double* y, int precision) {
    size_t hb = (size_t)ctx->n * ctx->P * sizeof(double);
    SG_TRY(sg_ensure(ctx, ctx->w_stage, hb));
    SG_TRY(sg_launch_from_device(ctx, src, (double*)ctx->w_stage.p, precision));
    SG_CUDA(ctx, cudaMemcpyAsync(y, ctx->w_stage.p, hb, cudaMemcpyDeviceToHost, ctx->stream));
    SG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return SGFEM_OK;
}

extern "C" int sgfem_device_layout(const sgfem_context* ctx, int64_t* n_dev, int64_t* ld) {
    if (!ctx || !ctx->finalized) return SGFEM_ERR_STATE;
    if (n_dev) *n_dev = ctx->n;
    if (ld) *ld = ctx->ld;
    return SGFEM_OK;
}

extern "C" int sgfem_to_device_layout(sgfem_context* ctx, const double* x_host, void* x_dev, int precision) {
    SG_TRY(sg_check_ready(ctx));
    SG_TRY(check_precision(ctx, precision));
    if (!x_host || !x_dev) return sg_fail(ctx, SGFEM_ERR_ARGUMENT, "null pointer");
    SG_CUDA(ctx, cudaSetDevice(ctx->device));
    SG_TRY(host_to_device_layout(ctx, x_host, x_dev, precision));
    SG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return SGFEM_OK;
}

extern "C" int sgfem_from_device_layout(sgfem_context* ctx, const void* x_dev, double* x_host, int precision) {
    SG_TRY(sg_check_ready(ctx));
    SG_TRY(check_precision(ctx, precision));
    if (!x_host || !x_dev) return sg_fail(ctx, SGFEM_ERR_ARGUMENT, "null pointer");
    SG_CUDA(ctx, cudaSetDevice(ctx->device));
    return device_to_host_layout(ctx, x_dev, x_host, precision);
}

extern "C" int sgfem_apply(sgfem_context* ctx, const double* x, double* y, int precision) {
    SG_TRY(sg_check_ready(ctx));
    SG_TRY(check_precision(ctx, precision));
    if (!x || !y) return sg_fail(ctx, SGFEM_ERR_ARGUMENT, "null pointer");
    SG_CUDA(ctx, cudaSetDevice(ctx->device));
    if (precision == SGFEM_FP32) SG_TRY(sg_jit_ensure(ctx));
    size_t vb = sg_vec_bytes(ctx, precision);
    SG_TRY(sg_ensure(ctx, ctx->w_vec[0], vb));
    SG_TRY(sg_ensure(ctx, ctx->w_vec[1], vb));
    SG_TRY(host_to_device_layout(ctx, x, ctx->w_vec[0].p, precision));
    SG_TRY(sg_launch_apply(ctx, precision, ctx->w_vec[0].p, ctx->w_vec[1].p, nullptr, nullptr, nullptr));
    if (precision == SGFEM_FP32) SG_TRY(sg_jit_check(ctx));
    return device_to_host_layout(ctx, ctx->w_vec[1].p, y, precision);
}

extern "C" int sgfem_apply_device(sgfem_context* ctx, const void* x_dev, void* y_dev, int precision) {
    SG_TRY(sg_check_ready(ctx));
    SG_TRY(check_precision(ctx, precision));
    if (!x_dev || !y_dev) return sg_fail(ctx, SGFEM_ERR_ARGUMENT, "null pointer");
    SG_CUDA(ctx, cudaSetDevice(ctx->device));
    if (precision == SGFEM_FP32) SG_TRY(sg_jit_ensure(ctx));
    SG_TRY(sg_launch_apply(ctx, precision, x_dev, y_dev, nullptr, nullptr, nullptr));
    SG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (precision == SGFEM_FP32) SG_TRY(sg_jit_check(ctx));
    return SGFEM_OK;
}

extern "C" int sgfem_time_apply(sgfem_context* ctx, int precision, int reps, double* ms_per_apply) {
    SG_TRY(sg_check_ready(ctx));
    SG_TRY(check_precision(ctx, precision));
    if (reps <= 0 || !ms_per_apply) return sg_fail(ctx, SGFEM_ERR_ARGUMENT, "bad reps");
    SG_CUDA(ctx, cudaSetDevice(ctx->device));
    if (precision == SGFEM_FP32) SG_TRY(sg_jit_ensure(ctx));
    size_t vb = sg_vec_bytes(ctx, precision);
    SG_TRY(sg_ensure(ctx, ctx->w_vec[0], vb));
    SG_TRY(sg_ensure(ctx, ctx->w_vec[1], vb));
    SG_CUDA(ctx, cudaMemsetAsync(ctx->w_vec[0].p, 0, vb, ctx->stream));
    SG_TRY(sg_launch_apply(ctx, precision, ctx->w_vec[0].p, ctx->w_vec[1].p, nullptr, nullptr, nullptr));
    SG_CUDA(ctx, cudaEventRecord(ctx->ev0, ctx->stream));
    for (int r = 0; r < reps; ++r) {
        // alternate the roles so consecutive launches do not reuse one output in L2
        const void* xin = (r & 1) ? ctx->w_vec[1].p : ctx->w_vec[0].p;
        void* yout = (r & 1) ? ctx->w_vec[0].p : ctx->w_vec[1].p;
        SG_TRY(sg_launch_apply(ctx, precision, xin, yout, nullptr, nullptr, nullptr));
    }
    SG_CUDA(ctx, cudaEventRecord(ctx->ev1, ctx->stream));
    SG_CUDA(ctx, cudaEventSynchronize(ctx->ev1));
    float ms = 0.f;
    SG_CUDA(ctx, cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
    *ms_per_apply = ms / reps;
    if (precision == SGFEM_FP32) SG_TRY(sg_jit_check(ctx));
    return SGFEM_OK;
}
