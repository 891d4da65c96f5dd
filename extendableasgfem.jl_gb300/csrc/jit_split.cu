// Specialised FP32 SG apply, split-slot form of the lattice-window kernel
// (compiled at the first FP32 use with NVRTC, like the forms in jit.cu; the
// operator of mul!, src/modelproblems/solvers_poisson_primal.jl:86-124).
//
//   F(m, c) = sum_j K_m[i, j] (x_j[c] - x_i[c])       (difference form)
//   Y[i, mu] = F(0, mu) + sum_{(m, nu)} G[(m-1)P + mu, nu] F(m, nu)
//
// Lane L owns the device columns c = 32 k + L (register k).  Two nonzeros are
// processed by one packed FP32x2 FMA: the accumulator (a.x, a.y) collects the
// even and the odd nonzeros of the row, the KLE values of a term for
// nonzeros (t, t+1) are adjacent in the row's staged value block (m-major:
// row m of the block holds K_m of the row's nonzeros), and the X values of a
// column for the two nonzeros form the other operand.  Three kinds of slots:
//   dense slot (m, k):  m warp-uniform (the KLE terms coupled to most columns),
//                       its values one broadcast load per four nonzeros;
//   own slot (k):       every lane its own term m(L) for its column 32 k + L,
//                       the values loaded per lane (the block rows are skewed
//                       so that different m fall into different banks);
//   shuffled slot (k):  every lane a term and a column 32 k + src(L) of another
//                       lane, whose (x_t, x_t+1) difference it fetches by two
//                       shuffles: the items of heavily coupled columns that own
//                       slots would pad.
// After the row the slot accumulators go to shared memory and each lane forms
// its share of the output columns by the combination list (as in jit.cu).
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>

#include "sgfem_internal.h"

namespace {
// floats per staged value row: 32 nonzeros plus a skew that puts rows m and m' in
// different 16-byte bank groups whenever m != m' (mod 8): 44 = 11 * 4, 11 odd
constexpr int KSTR = 44;
}

struct SplitApply {
    std::vector<int> dense_m;                   // dense KLE terms
    std::vector<std::pair<int, int>> dslots;    // (index into dense_m, register k)
    std::vector<int> own_k, sh_k;               // register of each own / shuffled slot
    std::vector<int> lanetab;                   // per sparse slot and lane: m * KSTR | src << 16
    std::vector<int2> jtab;                     // combination entries [T][32]
    int T = 0;                                  // combination entries per lane
    int cmax = 0;                               // longest row (nonzeros)
    int* d_lanetab = nullptr;
    int2* d_jtab = nullptr;
    double cost = 0.0;                          // modelled issue slots per nonzero
};

namespace {

struct Item {
    int m, c;
};

// modelled issue slots per nonzero of the loop body (see the header comment)
double model_cost(int KG, int nd, int nds, int nown, int nsh) {
    return 5.0 + 0.25 + 0.5 * KG + 0.25 * nd + 0.5 * nds + 0.75 * nown + 1.75 * nsh + 1.0;
}

}  // namespace

int sg_split_plan(sgfem_context* ctx, std::string& why) {
    sg_split_release(ctx);
    const int P = (int)ctx->P, M1 = ctx->M1, LD = (int)ctx->ld;
    const int KG = (P + 31) / 32;
    if (ctx->h_qtab.empty() || (int)ctx->h_combptr.size() != P + 1) {
        why = "coupling lists missing";
        return SGFEM_ERR_UNSUPPORTED;
    }
    if (M1 + 1 > 64 || P > 4096 || LD % 2) {
        why = "outside the split form's range";
        return SGFEM_ERR_UNSUPPORTED;
    }
    // longest row: at most 32 nonzeros (one staged block per row)
    const int cmax = ctx->row_nnz_max;
    if (cmax > 32 || cmax < 0) {
        why = "rows with more than 32 nonzeros";
        return SGFEM_ERR_UNSUPPORTED;
    }
    // pairs (m, c) of the operator, per term
    std::vector<std::vector<char>> inq(M1, std::vector<char>(P, 0));
    for (int32_t q : ctx->h_qtab) inq[q >> 16][q & 0xffff] = 1;
    std::vector<int> size(M1, 0);
    for (int m = 0; m < M1; ++m)
        for (int c = 0; c < P; ++c) size[m] += inq[m][c];
    std::vector<int> morder(M1);
    std::iota(morder.begin(), morder.end(), 0);
    std::stable_sort(morder.begin(), morder.end(), [&](int a, int b) {
        if ((a == 0) != (b == 0)) return a == 0;
        return size[a] > size[b];
    });

    struct Choice {
        double cost = 1e30;
        int nd = 0;
        std::vector<int> nown;  // own slots per register
    } best;
    // per register k and lane L: sparse items of column 32 k + L, for a dense count nd
    auto sparse_counts = [&](int nd, std::vector<std::vector<int>>& cnt) {
        std::vector<char> isdense(M1, 0);
        for (int d = 0; d < nd; ++d) isdense[morder[d]] = 1;
        cnt.assign(KG, std::vector<int>(32, 0));
        for (int m = 0; m < M1; ++m)
            if (!isdense[m])
                for (int c = 0; c < P; ++c)
                    if (inq[m][c]) cnt[c / 32][c % 32]++;
    };
    for (int nd = 1; nd <= std::min(M1, 8); ++nd) {
        int nds = 0;
        for (int d = 0; d < nd; ++d)
            for (int k = 0; k < KG; ++k) {
                bool any = false;
                for (int c = 32 * k; c < std::min(P, 32 * k + 32) && !any; ++c) any = inq[morder[d]][c];
                nds += any;
            }
        std::vector<std::vector<int>> cnt;
        sparse_counts(nd, cnt);
        int nown = 0, nsh = 0;
        std::vector<int> ownk(KG, 0);
        for (int k = 0; k < KG; ++k) {
            const int mx = *std::max_element(cnt[k].begin(), cnt[k].end());
            double bc = 1e30;
            int bn = 0, bsh = 0;
            for (int o = 0; o <= mx; ++o) {
                int left = 0;
                for (int L = 0; L < 32; ++L) left += std::max(0, cnt[k][L] - o);
                const int sh = (left + 31) / 32;
                const double c = 0.75 * o + 1.75 * sh;
                if (c < bc) {
                    bc = c;
                    bn = o;
                    bsh = sh;
                }
            }
            ownk[k] = bn;
            nown += bn;
            nsh += bsh;
        }
        // accumulator registers: two per slot; keep the total within reach of 16 warps per SM
        if (2 * (nds + nown + nsh) > 72) continue;
        const double cost = model_cost(KG, nd, nds, nown, nsh);
        if (cost < best.cost) {
            best.cost = cost;
            best.nd = nd;
            best.nown = ownk;
        }
    }
    if (best.nd == 0) {
        why = "too many slots for the split form";
        return SGFEM_ERR_UNSUPPORTED;
    }
    SplitApply* sp = new SplitApply();
    ctx->split = sp;
    sp->cost = best.cost;
    sp->cmax = cmax;
    (void)LD;
    const int nd = best.nd;
    std::vector<char> isdense(M1, 0);
    for (int d = 0; d < nd; ++d) {
        sp->dense_m.push_back(morder[d]);
        isdense[morder[d]] = 1;
    }
    // slot of F(m, c): offset slot * 32 + lane in the accumulator block
    std::vector<std::vector<int>> off(M1, std::vector<int>(P, -1));
    for (int d = 0; d < nd; ++d)
        for (int k = 0; k < KG; ++k) {
            bool any = false;
            for (int c = 32 * k; c < std::min(P, 32 * k + 32) && !any; ++c) any = inq[morder[d]][c];
            if (!any) continue;
            const int s = (int)sp->dslots.size();
            sp->dslots.push_back({d, k});
            for (int c = 32 * k; c < std::min(P, 32 * k + 32); ++c)
                if (inq[morder[d]][c]) off[morder[d]][c] = s * 32 + (c % 32);
        }
    const int NDS = (int)sp->dslots.size();
    // sparse items per lane of each register; own slots take them in an order that
    // spreads m mod 8 over each quarter warp (the banks of the per-lane value loads)
    struct SparseSlot {
        int k;
        bool own;
        Item it[32];
    };
    std::vector<SparseSlot> sslots;
    for (int k = 0; k < KG; ++k) {
        std::vector<std::vector<Item>> items(32);
        for (int L = 0; L < 32; ++L) {
            const int c = 32 * k + L;
            if (c >= P) continue;
            for (int m = 0; m < M1; ++m)
                if (!isdense[m] && inq[m][c]) items[L].push_back({m, c});
        }
        for (int j = 0; j < best.nown[k]; ++j) {
            SparseSlot ss;
            ss.k = k;
            ss.own = true;
            for (int ph = 0; ph < 4; ++ph) {
                unsigned used = 0;
                for (int L = 8 * ph; L < 8 * ph + 8; ++L) {
                    ss.it[L] = {-1, -1};
                    if (items[L].empty()) continue;
                    size_t pick = 0;
                    for (size_t q = 0; q < items[L].size(); ++q)
                        if (!(used & (1u << (items[L][q].m & 7)))) {
                            pick = q;
                            break;
                        }
                    ss.it[L] = items[L][pick];
                    used |= 1u << (items[L][pick].m & 7);
                    items[L].erase(items[L].begin() + pick);
                }
            }
            sslots.push_back(ss);
        }
        std::vector<Item> left;
        for (int L = 0; L < 32; ++L) left.insert(left.end(), items[L].begin(), items[L].end());
        while (!left.empty()) {
            SparseSlot ss;
            ss.k = k;
            ss.own = false;
            for (int ph = 0; ph < 4; ++ph) {
                unsigned used = 0;
                for (int L = 8 * ph; L < 8 * ph + 8; ++L) {
                    ss.it[L] = {-1, -1};
                    if (left.empty()) continue;
                    size_t pick = 0;
                    for (size_t q = 0; q < left.size(); ++q)
                        if (!(used & (1u << (left[q].m & 7)))) {
                            pick = q;
                            break;
                        }
                    ss.it[L] = left[pick];
                    used |= 1u << (left[pick].m & 7);
                    left.erase(left.begin() + pick);
                }
            }
            sslots.push_back(ss);
        }
    }
    // own slots first, then shuffled (the generated code walks them in this order)
    std::stable_sort(sslots.begin(), sslots.end(), [](const SparseSlot& a, const SparseSlot& b) {
        return a.own && !b.own;
    });
    sp->lanetab.assign(std::max<size_t>(1, sslots.size()) * 32, M1 * KSTR);
    for (size_t q = 0; q < sslots.size(); ++q) {
        const SparseSlot& ss = sslots[q];
        (ss.own ? sp->own_k : sp->sh_k).push_back(ss.k);
        const int s = NDS + (int)q;
        for (int L = 0; L < 32; ++L) {
            const Item& it = ss.it[L];
            if (it.m < 0) {  // padding: the zero row of the staged block, own lane as source
                sp->lanetab[q * 32 + L] = M1 * KSTR | (L << 16);
                continue;
            }
            const int src = it.c % 32;
            sp->lanetab[q * 32 + L] = it.m * KSTR | (src << 16);
            off[it.m][it.c] = s * 32 + L;
        }
    }
    const int NSL = NDS + (int)sslots.size();
    if (NSL * 32 >= 8192) {
        why = "accumulator block too large";
        sg_split_release(ctx);
        return SGFEM_ERR_UNSUPPORTED;
    }
    // combination: per output column (1, F(0, c)) then (g, F(m, nu)); columns to the
    // least loaded lane, longest lists first
    std::vector<std::vector<std::pair<int, float>>> colent(P);
    for (int c = 0; c < P; ++c) {
        if (off[0][c] < 0) {
            why = "internal: F(0, c) without a slot";
            sg_split_release(ctx);
            return SGFEM_ERR_UNSUPPORTED;
        }
        colent[c].push_back({off[0][c], 1.0f});
        for (int32_t e = ctx->h_combptr[c]; e < ctx->h_combptr[c + 1]; ++e) {
            const int32_t q = ctx->h_qtab[ctx->h_combq[e]];
            const int m = q >> 16, nu = q & 0xffff;
            if (off[m][nu] < 0) {
                why = "internal: coupling without a slot";
                sg_split_release(ctx);
                return SGFEM_ERR_UNSUPPORTED;
            }
            colent[c].push_back({off[m][nu], (float)ctx->h_combg[e]});
        }
    }
    std::vector<int> order(P);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return colent[a].size() > colent[b].size(); });
    std::vector<std::vector<int2>> lanes(32);
    std::vector<size_t> load(32, 0);
    for (int c : order) {
        int bl = 0;
        for (int L = 1; L < 32; ++L)
            if (load[L] < load[bl]) bl = L;
        load[bl] += colent[c].size();
        for (size_t e = 0; e < colent[c].size(); ++e) {
            int bits;
            std::memcpy(&bits, &colent[c][e].second, sizeof(int));
            const bool last = e + 1 == colent[c].size();
            lanes[bl].push_back(make_int2(colent[c][e].first | (c << 13) | ((last ? 1 : 0) << 28), bits));
        }
    }
    size_t T = 0;
    for (auto& l : lanes) T = std::max(T, l.size());
    if (T == 0 || T > 256) {
        why = "combination list too long";
        sg_split_release(ctx);
        return SGFEM_ERR_UNSUPPORTED;
    }
    sp->T = (int)T;
    sp->jtab.assign(T * 32, make_int2(0, 0));  // padding entries: g = 0, no output
    for (int L = 0; L < 32; ++L)
        for (size_t i = 0; i < lanes[L].size(); ++i) sp->jtab[i * 32 + L] = lanes[L][i];
    return SGFEM_OK;
}

int sg_split_upload(sgfem_context* ctx) {
    SplitApply* sp = ctx->split;
    if (cudaMalloc((void**)&sp->d_jtab, sp->jtab.size() * sizeof(int2)) != cudaSuccess ||
        cudaMemcpy(sp->d_jtab, sp->jtab.data(), sp->jtab.size() * sizeof(int2), cudaMemcpyHostToDevice) !=
            cudaSuccess ||
        cudaMalloc((void**)&sp->d_lanetab, sp->lanetab.size() * sizeof(int)) != cudaSuccess ||
        cudaMemcpy(sp->d_lanetab, sp->lanetab.data(), sp->lanetab.size() * sizeof(int), cudaMemcpyHostToDevice) !=
            cudaSuccess)
        return SGFEM_ERR_CUDA;
    return SGFEM_OK;
}

size_t sg_split_smem(const sgfem_context* ctx, int wpb) {
    const SplitApply* sp = ctx->split;
    const size_t W = (size_t)wpb * ctx->jit_wrw, SW = W + 2 * (size_t)ctx->win_hx, WL = 2 * (size_t)ctx->win_hy + 2;
    const size_t KB = (size_t)(ctx->M1 + 1) * KSTR;
    const size_t NSL = sp->dslots.size() + sp->own_k.size() + sp->sh_k.size();
    const size_t sacc = NSL * 32 > KB ? NSL * 32 : 0;
    const size_t wsmem = 2 * KB + sacc + (((size_t)ctx->ld + 3) & ~(size_t)3) + 32;
    return (2 * (size_t)sp->T * 32 + WL * SW * ctx->ld + wpb * wsmem) * sizeof(float);
}

const int* sg_split_lanetab(const sgfem_context* ctx) { return ctx->split ? ctx->split->d_lanetab : nullptr; }

const int2* sg_split_jtab(const sgfem_context* ctx) { return ctx->split ? ctx->split->d_jtab : nullptr; }

std::string sg_split_summary(const sgfem_context* ctx) {
    const SplitApply* sp = ctx->split;
    if (!sp) return "";
    char b[256];
    snprintf(b, sizeof(b), "split slots: %zu dense (%zu terms) + %zu own + %zu shuffled, %d combination entries/lane",
             sp->dslots.size(), sp->dense_m.size(), sp->own_k.size(), sp->sh_k.size(), sp->T);
    return b;
}

void sg_split_release(sgfem_context* ctx) {
    SplitApply* sp = ctx->split;
    if (!sp) return;
    if (sp->d_jtab) cudaFree(sp->d_jtab);
    if (sp->d_lanetab) cudaFree(sp->d_lanetab);
    delete sp;
    ctx->split = nullptr;
}

std::string sg_split_source(const sgfem_context* ctx) {
    const SplitApply* sp = ctx->split;
    const int LD = (int)ctx->ld, P = (int)ctx->P, M1 = ctx->M1, M1P = ctx->M1P;
    const int KG = (P + 31) / 32;
    const int NDS = (int)sp->dslots.size(), NOWN = (int)sp->own_k.size(), NSH = (int)sp->sh_k.size();
    const int NSL = NDS + NOWN + NSH;
    const int ND = (int)sp->dense_m.size();
    std::string s;
    char buf[768];
    snprintf(buf, sizeof(buf),
             "#define LD %d\n#define P %d\n#define KG %d\n#define M1 %d\n#define M1P %d\n#define KSTR %d\n"
             "#define NSL %d\n#define NSP %d\n#define WPB %d\n#define T %d\n#define DIFF %d\n#define NLX %d\n"
             "#define NLY %d\n#define HX %d\n#define HY %d\n#define RW %d\n",
             LD, P, KG, M1, M1P, KSTR, NSL, NOWN + NSH, ctx->jit_wwpb, sp->T, ctx->jit_diff, ctx->lat_np,
             ctx->lat_np, ctx->win_hx, ctx->win_hy, ctx->jit_wrw);
    s += buf;
    s += R"(
#define NV4 (M1P / 4)
#define W (WPB * RW)
#define SW (W + 2 * HX)
#define WL (2 * HY + 2)
#define NSTRIP ((NLX + W - 1) / W)
#define LINES (NSTRIP * NLY)
#define KB ((M1 + 1) * KSTR)              /* staged values of one row, m-major, plus a zero row */
#define SACC (NSL * 32 > KB ? NSL * 32 : 0)          /* in the row's staged block, or separate */
#define WSMEM (2 * KB + SACC + ((LD + 3) & ~3) + 32)  /* two staged blocks (current, next row) */
#define WIN (WL * SW * LD)
struct Scal { double rho, pq, alpha, beta, rr, tol2; int done, status, iters, first; };

__device__ __forceinline__ void cp16(float* dst, const float* src) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_wait_all() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }

__device__ __forceinline__ void copy_line(float* win, const float* __restrict__ X, int ly, int xs) {
    const int cx0 = max(0, xs), cx1 = min(NLX, xs + SW);
    const int n4 = (cx1 - cx0) * (LD / 4);
    const float* src = X + ((size_t)ly * NLX + cx0) * LD;
    float* dst = win + ((ly % WL) * SW + (cx0 - xs)) * LD;
    for (int i = threadIdx.x; i < n4; i += WPB * 32) cp16(dst + 4 * i, src + 4 * i);
}

// the values of a row's nonzeros (nonzero-major in global memory, M1P per nonzero)
// into a staged block, transposed to m-major (row m at m * KSTR), one 4-byte
// cp.async per value
__device__ __forceinline__ void stage_values(float* kbuf, const float* __restrict__ vals, int nz0, int cnt, int lane) {
    const unsigned d0 = (unsigned)__cvta_generic_to_shared(kbuf);
    for (int q = lane; q < cnt * M1; q += 32) {
        const int t = q / M1, m = q - t * M1;
        const float* src = vals + (size_t)(nz0 + t) * M1P + m;
        asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(d0 + 4u * (unsigned)(m * KSTR + t)), "l"(src)
                     : "memory");
    }
}

__device__ __forceinline__ int seg_row(int k, int ya, int x0, int warp) {
    const int x = x0 + warp * RW + k % RW;
    return x < NLX ? (ya + k / RW) * NLX + x : -1;
}

extern "C" __global__ void __launch_bounds__(WPB * 32, 1)
sg_apply_jit(const int* __restrict__ rowptr, const int* __restrict__ col, const float* __restrict__ vals,
             const float* __restrict__ X, float* __restrict__ Y, int n, const unsigned char* __restrict__ bmask,
             const int2* __restrict__ jtab, const int* __restrict__ lanetab, double* __restrict__ partials,
             const Scal* __restrict__ scal, int* __restrict__ err) {
    if (scal && scal->done) return;
    extern __shared__ __align__(16) float smem[];
    __shared__ double red[WPB];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    int2* stab = reinterpret_cast<int2*>(smem);
    float* win = smem + 2 * T * 32;
    float* wb = win + WIN + warp * WSMEM;
    float* kbs = wb;                                  // staged values: current and next row
    float* sacc0 = wb + 2 * KB;                       // slot accumulators when they do not fit below the zero row
    float* ybuf = wb + 2 * KB + SACC;
    int* offs = reinterpret_cast<int*>(ybuf + ((LD + 3) & ~3));
    for (int i = threadIdx.x; i < T * 32; i += blockDim.x) stab[i] = __ldg(jtab + i);
    kbs[M1 * KSTR + lane] = 0.f;                     // zero rows (padding lanes of sparse slots)
    kbs[KB + M1 * KSTR + lane] = 0.f;
    int cur = 0;
)";
    // per-lane sparse slot parameters
    for (int q = 0; q < NOWN + NSH; ++q) {
        snprintf(buf, sizeof(buf), "    const int lt%d = __ldg(lanetab + %d * 32 + lane);\n", q, q);
        s += buf;
        if (q >= NOWN) {
            snprintf(buf, sizeof(buf), "    const int src%d = lt%d >> 16;\n", q, q);
            s += buf;
        }
        snprintf(buf, sizeof(buf), "    const int ko%d = lt%d & 0xffff;\n", q, q);
        s += buf;
    }
    s += R"(    double dot = 0.0;
    int bad = 0;
    const int g0 = (int)(((long long)blockIdx.x * LINES) / gridDim.x);
    const int g1 = (int)(((long long)(blockIdx.x + 1) * LINES) / gridDim.x);
    for (int g = g0; g < g1;) {
        const int strip = g / NLY, ya = g - strip * NLY;
        const int yb = min(NLY, ya + (g1 - g));
        g += yb - ya;
        const int x0 = strip * W, xs = x0 - HX;
        __syncthreads();
        for (int ly = max(0, ya - HY); ly <= min(NLY - 1, ya + HY); ++ly) copy_line(win, X, ly, xs);
        cp_commit();
        const int KR = (yb - ya) * RW;
        int k = 0;
        while (k < KR && seg_row(k, ya, x0, warp) < 0) ++k;
        int jn1 = 0, cn1 = 0;
        if (k < KR) {  // the warp's first row: its columns, its values staged
            const int r0 = seg_row(k, ya, x0, warp);
            const int a = __ldg(rowptr + r0);
            cn1 = __ldg(rowptr + r0 + 1) - a;
            jn1 = (lane < cn1) ? __ldg(col + a + lane) : 0;
            __syncwarp();
            stage_values(kbs + cur * KB, vals, a, cn1, lane);
            cp_commit();
        }
        for (int kk = 0; kk < KR; ++kk) {
            // this row's staged values and (at a line start) the window lines it needs; the
            // copies issued below (the next line, the next row's values) stay in flight
            cp_wait_all();
            if (kk % RW == 0) {
                const int y = ya + kk / RW;
                __syncthreads();
                if (y + HY + 1 < NLY && y + 1 < yb) copy_line(win, X, y + HY + 1, xs);
                cp_commit();
            }
            const int row = seg_row(kk, ya, x0, warp);
            if (row < 0) continue;
            const int y = ya + kk / RW, x = row - y * NLX;
            const int jcur = jn1, cnt = cn1;
            float* kb = kbs + cur * KB;
            if ((cnt & 1) && lane < M1) kb[lane * KSTR + cnt] = 0.f;  // complete the last pair
            int kn = kk + 1;
            while (kn < KR && seg_row(kn, ya, x0, warp) < 0) ++kn;
            const int r1n = kn < KR ? seg_row(kn, ya, x0, warp) : -1;
            if (r1n >= 0) {  // next row: columns, and its values staged into the other block
                const int a = __ldg(rowptr + r1n);
                cn1 = __ldg(rowptr + r1n + 1) - a;
                jn1 = (lane < cn1) ? __ldg(col + a + lane) : 0;
                stage_values(kbs + (cur ^ 1) * KB, vals, a, cn1, lane);
                cp_commit();
            }
            float* sacc = SACC ? sacc0 : kb;
            float* yrow = Y + (size_t)row * LD;
            const float* xown = win + ((y % WL) * SW + (x - xs)) * LD;
            __syncwarp();
            if (bmask[row]) {
                for (int c = lane; c < LD; c += 32) yrow[c] = 0.f;
            } else {
                // window offset of each nonzero (padding: the row itself, so x_j - x_i = 0)
                {
                    int o = (int)(xown - win);
                    if (lane < cnt) {
                        const int cy = jcur / NLX, cx = jcur - cy * NLX;
                        const int dy = cy - y, wx = cx - xs;
                        if (dy < -HY || dy > HY || wx < 0 || wx >= SW) bad = 1;
                        else o = ((cy % WL) * SW + wx) * LD;
                    }
                    offs[lane] = o;
                }
                __syncwarp();
)";
    // own-row values, negated and duplicated (difference form)
    for (int k = 0; k < KG; ++k) {
        const int valid = LD - 32 * k;
        if (valid >= 32)
            snprintf(buf, sizeof(buf), "                const float xi%d = DIFF ? -xown[%d + lane] : 0.f;\n", k, 32 * k);
        else
            snprintf(buf, sizeof(buf), "                const float xi%d = (DIFF && lane < %d) ? -xown[%d + lane] : 0.f;\n",
                     k, valid, 32 * k);
        s += buf;
        snprintf(buf, sizeof(buf), "                const float2 nx%d = make_float2(xi%d, xi%d);\n", k, k, k);
        s += buf;
    }
    for (int q = 0; q < NSL; ++q) {
        snprintf(buf, sizeof(buf), "                float2 a%d = make_float2(0.f, 0.f);\n", q);
        s += buf;
    }
    // u<k>_<h> = (x_t - x_i, x_t+1 - x_i) of column 32 k + lane for the pair h of the step
    auto upair = [&](const char* h) {
        std::string b;
        char l[512];
        for (int k = 0; k < KG; ++k) {
            const int valid = LD - 32 * k;
            if (valid >= 32)
                snprintf(l, sizeof(l),
                         "                    const float2 u%d_%s = __fadd2_rn(make_float2(win[o0_%s + %d + lane], "
                         "win[o1_%s + %d + lane]), nx%d);\n",
                         k, h, h, 32 * k, h, 32 * k, k);
            else
                snprintf(l, sizeof(l),
                         "                    const float2 u%d_%s = (lane < %d) ? __fadd2_rn(make_float2(win[o0_%s + %d "
                         "+ lane], win[o1_%s + %d + lane]), nx%d) : make_float2(0.f, 0.f);\n",
                         k, h, valid, h, 32 * k, h, 32 * k, k);
            b += l;
        }
        return b;
    };
    // the slots for the pairs of the step: values loaded slot by slot (four nonzeros per
    // float4 in a full step, two per float2 in the last pair) and used at once
    auto slots = [&](bool full) {
        std::string b;
        char l[768];
        for (int d = 0; d < ND; ++d) {
            if (full)
                snprintf(l, sizeof(l), "                    { const float4 kv = *reinterpret_cast<const float4*>(kb + %d * KSTR + t);\n",
                         sp->dense_m[d]);
            else
                snprintf(l, sizeof(l), "                    { const float2 kv = *reinterpret_cast<const float2*>(kb + %d * KSTR + t);\n",
                         sp->dense_m[d]);
            b += l;
            for (int q = 0; q < NDS; ++q) {
                if (sp->dslots[q].first != d) continue;
                const int k = sp->dslots[q].second;
                snprintf(l, sizeof(l), "                      a%d = __ffma2_rn(make_float2(kv.x, kv.y), u%d_0, a%d);\n", q, k, q);
                b += l;
                if (full) {
                    snprintf(l, sizeof(l), "                      a%d = __ffma2_rn(make_float2(kv.z, kv.w), u%d_1, a%d);\n", q, k, q);
                    b += l;
                }
            }
            b += "                    }\n";
        }
        for (int q = 0; q < NOWN + NSH; ++q) {
            const bool sh = q >= NOWN;
            const int k = sh ? sp->sh_k[q - NOWN] : sp->own_k[q];
            const int a = NDS + q;
            if (full)
                snprintf(l, sizeof(l), "                    { const float4 kw = *reinterpret_cast<const float4*>(kb + ko%d + t);\n", q);
            else
                snprintf(l, sizeof(l), "                    { const float2 kw = *reinterpret_cast<const float2*>(kb + ko%d + t);\n", q);
            b += l;
            for (int h = 0; h < (full ? 2 : 1); ++h) {
                const char* kx = h ? "kw.z, kw.w" : "kw.x, kw.y";
                if (!sh)
                    snprintf(l, sizeof(l), "                      a%d = __ffma2_rn(make_float2(%s), u%d_%d, a%d);\n", a, kx, k, h, a);
                else
                    snprintf(l, sizeof(l),
                             "                      a%d = __ffma2_rn(make_float2(%s), make_float2(__shfl_sync(0xffffffffu, u%d_%d.x, "
                             "src%d), __shfl_sync(0xffffffffu, u%d_%d.y, src%d)), a%d);\n",
                             a, kx, k, h, q, k, h, q, a);
                b += l;
            }
            b += "                    }\n";
        }
        return b;
    };
    // full steps of four nonzeros
    s += "                const int cnt2 = (cnt + 1) & ~1;\n";
    s += "                int t = 0;\n";
    s += "                for (; t + 4 <= cnt2; t += 4) {\n";
    s += "                    const int4 oo = *reinterpret_cast<const int4*>(offs + t);\n";
    s += "                    const int o0_0 = oo.x, o1_0 = oo.y, o0_1 = oo.z, o1_1 = oo.w;\n";
    s += upair("0");
    s += upair("1");
    s += slots(true);
    s += "                }\n";
    // a remaining pair
    s += "                if (t < cnt2) {\n";
    s += "                    const int2 oo = *reinterpret_cast<const int2*>(offs + t);\n";
    s += "                    const int o0_0 = oo.x, o1_0 = oo.y;\n";
    s += upair("0");
    s += slots(false);
    s += "                }\n";
    s += "                __syncwarp();  // staged values read: their storage may take the accumulators\n";
    for (int q = 0; q < NSL; ++q) {
        snprintf(buf, sizeof(buf), "                sacc[%d * 32 + lane] = a%d.x + a%d.y;\n", q, q, q);
        s += buf;
    }
    s += R"(                __syncwarp();
                float acc = 0.f;
#pragma unroll 4
                for (int i = 0; i < T; ++i) {
                    const int2 e = stab[i * 32 + lane];
                    acc = fmaf(__int_as_float(e.y), sacc[e.x & 0x1fff], acc);
                    if (e.x >> 28) {
                        ybuf[(e.x >> 13) & 0x7fff] = acc;
                        acc = 0.f;
                    }
                }
                __syncwarp();
                if (!SACC && NSL * 32 > M1 * KSTR) kb[M1 * KSTR + lane] = 0.f;  // the accumulators covered the zero row
                float rowdot = 0.f;
                for (int c = lane; c < LD; c += 32) {
                    const float yv = (c < P) ? ybuf[c] : 0.f;
                    yrow[c] = yv;
                    if (partials) rowdot = fmaf(xown[c], yv, rowdot);
                }
                dot += (double)rowdot;
            }
            __syncwarp();  // accumulator reads done: this block may be staged again
            cur ^= 1;
        }
    }
    cp_wait_all();
    if (bad) atomicOr(err, 4);
    if (partials) {
        for (int o = 16; o > 0; o >>= 1) dot += __shfl_down_sync(0xffffffffu, dot, o);
        if (lane == 0) red[warp] = dot;
        __syncthreads();
        if (threadIdx.x == 0) {
            double t2 = 0.0;
            for (int w2 = 0; w2 < WPB; ++w2) t2 += red[w2];
            partials[blockIdx.x] = t2;
        }
    }
}
)";
    return s;
}
