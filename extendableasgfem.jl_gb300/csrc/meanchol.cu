// Mean-based preconditioner on any mesh: z = (I (x) K_0^-1) r on the interior
// rows, i.e. the reference's LU(K_0) solve of ldiv!
// (src/modelproblems/solvers_poisson_primal.jl:23-78: K_0 with 1e60 on the
// boundary diagonals, one solve per mode) for meshes whose dofs do not form a
// power-of-two lattice: the RGB-refined meshes of the adaptive loop
// (scripts/poisson.jl:395-405), perturbed or graded meshes.
//
// Host, once per context at the first use:
//   * nested-dissection ordering of the interior graph of K_0: a breadth-first
//     level structure rooted at a pseudo-peripheral vertex, its middle level is
//     a vertex separator of the rest; the two sides are ordered first
//     (recursively), the separator after them; pieces of at most kLeaf
//     vertices are leaves; disconnected pieces are split into components;
//   * up-looking sparse Cholesky K_0,II = L L^T in FP64 (elimination tree,
//     row patterns by tree reach, rows of L in order);
//   * for every node of the dissection tree (leaf or separator: a contiguous
//     range of rows of L) the dense inverse of its diagonal block of L.
// Device, per application (FP64 or FP32 values, lanes over modes, one warp per
// (row, 32 modes)): the forward solve L y = r visits the tree by height, leaves
// first; per height one gather launch t_k = r_k - sum_{j outside the node}
// L_kj y_j (those j lie in descendant nodes, already final) and one dense launch
// y_K = inv(L_KK) t_K.  The backward solve L^T z = y visits the heights root
// first with the columns of L (the rows of L^T) outside the node, which lie in
// ancestor nodes.  Rows of one height are independent; sums run in a fixed
// order, so results are bitwise reproducible.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>

#include "sgfem_internal.h"

namespace {

constexpr int kLeaf = 32;          // largest leaf of the dissection tree
constexpr int kWarps = 8;          // warps per block of the solve kernels

struct NDNode {
    int r0 = 0, r1 = 0;   // rows [r0, r1) of L (elimination order)
    int parent = -1;
    int height = 0;
};

// nested dissection by breadth-first level structures on the interior graph
struct Dissection {
    const std::vector<int64_t>& adjp;
    const std::vector<int32_t>& adji;
    std::vector<int32_t> stamp, dist, queue;
    std::vector<int32_t> order;  // elimination position -> interior vertex
    std::vector<NDNode> nodes;
    int cur = 0;

    Dissection(const std::vector<int64_t>& p, const std::vector<int32_t>& i, int64_t n)
        : adjp(p), adji(i), stamp(n, 0), dist(n, -1), queue(n) {
        order.reserve(n);
    }

    // BFS from s inside the vertices stamped `st`; returns the visit count, queue holds the order
    int64_t bfs(int32_t s, int st) {
        int64_t head = 0, tail = 0;
        queue[tail++] = s;
        dist[s] = 0;
        stamp[s] = -st;  // visited in this BFS
        while (head < tail) {
            const int32_t v = queue[head++];
            for (int64_t k = adjp[v]; k < adjp[v + 1]; ++k) {
                const int32_t w = adji[k];
                if (stamp[w] == st) {
                    stamp[w] = -st;
                    dist[w] = dist[v] + 1;
                    queue[tail++] = w;
                }
            }
        }
        return tail;
    }

    void leaf(int id, const std::vector<int32_t>& V) {
        nodes[id].r0 = (int)order.size();
        order.insert(order.end(), V.begin(), V.end());
        nodes[id].r1 = (int)order.size();
    }

    int build(std::vector<int32_t> V, int parent) {
        const int id = (int)nodes.size();
        nodes.push_back(NDNode{0, 0, parent, 0});
        if ((int64_t)V.size() <= kLeaf) {
            leaf(id, V);
            return id;
        }
        int st = ++cur;
        for (int32_t v : V) stamp[v] = st;
        int64_t cnt = bfs(V[0], st);
        if (cnt < (int64_t)V.size()) {  // disconnected: this node has no rows, two children
            std::vector<int32_t> A(queue.begin(), queue.begin() + cnt), B;
            B.reserve(V.size() - cnt);
            for (int32_t v : V)
                if (stamp[v] == st) B.push_back(v);
            build(std::move(A), id);
            build(std::move(B), id);
            nodes[id].r0 = nodes[id].r1 = (int)order.size();
            return id;
        }
        // pseudo-peripheral root: restart from the last vertex reached
        const int32_t u = queue[cnt - 1];
        st = ++cur;
        for (int32_t v : V) stamp[v] = st;
        cnt = bfs(u, st);
        const int h = dist[queue[cnt - 1]];
        if (h < 2) {  // no separating level: a dense leaf
            leaf(id, V);
            return id;
        }
        std::vector<int64_t> per(h + 1, 0);
        for (int32_t v : V) per[dist[v]]++;
        int m = 1;
        int64_t below = per[0];
        while (m < h - 1 && below + per[m] < (int64_t)V.size() / 2) below += per[m++];
        std::vector<int32_t> A, S, B;
        for (int64_t q = 0; q < cnt; ++q) {  // BFS order keeps neighbours close
            const int32_t v = queue[q];
            (dist[v] < m ? A : (dist[v] == m ? S : B)).push_back(v);
        }
        build(std::move(A), id);
        build(std::move(B), id);
        leaf(id, S);
        return id;
    }
};

}  // namespace

struct MeanChol {
    // K_0 on the interior rows, device numbering (kept until the factorisation)
    std::vector<int64_t> rowptr;
    std::vector<int32_t> col;
    std::vector<double> val;
    std::vector<int32_t> interior;  // interior index -> device row
    bool factored = false;
    int status = SGFEM_OK;
    std::string log = "not factored yet (at the first use)";
    int64_t ni = 0;
    int64_t nnzL = 0;
    size_t dinv_entries = 0;
    int nnodes = 0;
    std::vector<int> hptr;  // rows of height h: d_rows[hptr[h] .. hptr[h+1])
    // device
    int* d_dev = nullptr;      // elimination row -> device row
    int* d_rows = nullptr;     // rows grouped by height
    int* d_na = nullptr;       // per row: first row of its node
    int* d_ns = nullptr;       // per row: size of its node
    long long* d_noff = nullptr;  // per row: offset of its node's inverse block
    int* d_fptr = nullptr;     // forward gather: row k -> columns j < node start
    int* d_fcol = nullptr;
    double* d_fval64 = nullptr;
    float* d_fval32 = nullptr;
    int* d_bptr = nullptr;     // backward gather: column k -> rows i >= node end
    int* d_bcol = nullptr;
    double* d_bval64 = nullptr;
    float* d_bval32 = nullptr;
    double* d_dinv64 = nullptr;   // inv(L_KK), row-major s x s per node
    float* d_dinv32 = nullptr;
    double* d_dinvt64 = nullptr;  // its transpose
    float* d_dinvt32 = nullptr;
    int* d_brows = nullptr;    // boundary device rows (zeroed in the output)
    int nb = 0;
    DeviceBuf w_t, w_y;        // work vectors in elimination order, ni x ld
};

namespace {

template <typename T>
__global__ void k_chol_gather(const int* __restrict__ rows, int nrows, int nchunk, int ld, const int* __restrict__ ptr,
                              const int* __restrict__ idx, const T* __restrict__ val, const T* __restrict__ R,
                              const int* __restrict__ dev, const T* __restrict__ src, T* __restrict__ Tt,
                              const KrylovScalars* __restrict__ scal) {
    if (scal && scal->done) return;
    const int wid = (int)(blockIdx.x * kWarps + (threadIdx.x >> 5));
    const int lane = threadIdx.x & 31;
    if (wid >= nrows * nchunk) return;
    const int k = rows[wid / nchunk];
    const int c = (wid % nchunk) * 32 + lane;
    if (c >= ld) return;
    // forward: R is the device-layout right-hand side (dev maps the row); backward: R = src itself
    T acc = dev ? R[(size_t)dev[k] * ld + c] : src[(size_t)k * ld + c];
    for (int p = ptr[k]; p < ptr[k + 1]; ++p) acc -= val[p] * src[(size_t)idx[p] * ld + c];
    Tt[(size_t)k * ld + c] = acc;
}

template <typename T, bool BWD>
__global__ void k_chol_dense(const int* __restrict__ rows, int nrows, int nchunk, int ld, const int* __restrict__ na,
                             const int* __restrict__ ns, const long long* __restrict__ noff,
                             const T* __restrict__ dinv, const T* __restrict__ Tt, T* __restrict__ Y,
                             const int* __restrict__ dev, T* __restrict__ Z, const KrylovScalars* __restrict__ scal) {
    if (scal && scal->done) return;
    const int wid = (int)(blockIdx.x * kWarps + (threadIdx.x >> 5));
    const int lane = threadIdx.x & 31;
    if (wid >= nrows * nchunk) return;
    const int k = rows[wid / nchunk];
    const int c = (wid % nchunk) * 32 + lane;
    if (c >= ld) return;
    const int a = na[k], s = ns[k], r = k - a;
    const T* drow = dinv + noff[k] + (size_t)r * s;  // row r of inv(L_KK) (forward) or of its transpose
    T acc = T(0);
    if (!BWD) {
        for (int u = 0; u <= r; ++u) acc += drow[u] * Tt[(size_t)(a + u) * ld + c];
    } else {
        for (int u = r; u < s; ++u) acc += drow[u] * Tt[(size_t)(a + u) * ld + c];
    }
    Y[(size_t)k * ld + c] = acc;
    if (BWD) Z[(size_t)dev[k] * ld + c] = acc;
}

template <typename T>
__global__ void k_zero_rows(T* __restrict__ Z, const int* __restrict__ brows, int nb, int ld,
                            const KrylovScalars* __restrict__ scal) {
    if (scal && scal->done) return;
    const size_t total = (size_t)nb * ld;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x)
        Z[(size_t)brows[i / ld] * ld + i % ld] = T(0);
}

// mode 2: r'z partials over the interior rows; mode 1: P = Z + beta P on the interior rows
template <typename T>
__global__ void k_chol_finish(const T* __restrict__ R, const T* __restrict__ Z, T* __restrict__ P,
                              const unsigned char* __restrict__ bmask, int n, int ld, int mode,
                              double* __restrict__ rz, const KrylovScalars* __restrict__ scal) {
    if (scal && scal->done) return;
    __shared__ double red[8];
    T beta = T(0);
    if (mode == 1 && scal && !scal->first) beta = (T)scal->beta;
    T acc = T(0);
    const size_t total = (size_t)n * ld;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
        if (bmask[i / ld]) continue;
        if (mode == 2) acc = fma(R[i], Z[i], acc);
        else P[i] = Z[i] + beta * P[i];
    }
    if (mode == 2) {
        double a = (double)acc;
        for (int o = 16; o > 0; o >>= 1) a += __shfl_down_sync(0xffffffffu, a, o);
        if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = a;
        __syncthreads();
        if (threadIdx.x == 0) {
            double s = 0.0;
            for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += red[w];
            rz[blockIdx.x] = s;
        }
    }
}

template <typename T>
int upload_vec(sgfem_context* ctx, T** dst, const std::vector<T>& v) {
    const size_t bytes = std::max<size_t>(1, v.size()) * sizeof(T);
    SG_CUDA(ctx, cudaMalloc((void**)dst, bytes));
    if (!v.empty()) SG_CUDA(ctx, cudaMemcpy(*dst, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice));
    return SGFEM_OK;
}

std::vector<float> to_f32(const std::vector<double>& v) {
    std::vector<float> o(v.size());
    for (size_t i = 0; i < v.size(); ++i) o[i] = (float)v[i];
    return o;
}

// Everything the device solve needs, computed on the host (no CUDA calls): usable by
// the context (upload below) and by the host-only check entry point.
struct HostFactor {
    int64_t ni = 0, nnzL = 0;
    std::vector<int> dev, rows, na, ns, fptr, fcol, bptr, bcol, brows, hptr;
    std::vector<long long> noff;
    std::vector<double> fval, bval, dinv, dinvt;
    int nnodes = 0, H = 0, maxs = 0;
    std::string err;
};

// K_0 rows in device numbering (rowptr/col/val, interior rows only filled), interior
// index -> device row, boundary mask; returns SGFEM_OK or an error code with f.err
int host_factor(int64_t n, const std::vector<int64_t>& krowptr, const std::vector<int32_t>& kcol,
                const std::vector<double>& kval, const std::vector<int32_t>& interior,
                const std::vector<unsigned char>& bmask, HostFactor& f) {
    const int64_t ni = (int64_t)interior.size();
    f.ni = ni;
    std::vector<int32_t> iidx(n, -1);  // device row -> interior index
    for (int64_t i = 0; i < ni; ++i) iidx[interior[i]] = (int32_t)i;
    // interior graph without the diagonal
    std::vector<int64_t> adjp(ni + 1, 0);
    std::vector<int32_t> adji;
    adji.reserve(kcol.size());
    for (int64_t i = 0; i < ni; ++i) {
        const int32_t r = interior[i];
        for (int64_t k = krowptr[r]; k < krowptr[r + 1]; ++k) {
            const int32_t j = iidx[kcol[k]];
            if (j >= 0 && j != i && kval[k] != 0.0) adji.push_back(j);
        }
        adjp[i + 1] = (int64_t)adji.size();
    }
    // ---- ordering
    Dissection nd(adjp, adji, ni);
    if (ni > 0) {
        std::vector<int32_t> all(ni);
        std::iota(all.begin(), all.end(), 0);
        nd.build(std::move(all), -1);
    }
    const std::vector<int32_t>& order = nd.order;
    std::vector<int32_t> pos(ni);
    for (int64_t e = 0; e < ni; ++e) pos[order[e]] = (int32_t)e;
    std::vector<NDNode>& nodes = nd.nodes;
    for (int id = (int)nodes.size() - 1; id >= 0; --id)  // children have larger ids
        if (nodes[id].parent >= 0)
            nodes[nodes[id].parent].height = std::max(nodes[nodes[id].parent].height, nodes[id].height + 1);
    std::vector<int32_t> node_of(ni, -1);
    for (int id = 0; id < (int)nodes.size(); ++id)
        for (int e = nodes[id].r0; e < nodes[id].r1; ++e) node_of[e] = id;
    // ---- lower triangle of the permuted matrix, by rows: A'(k, j), j <= k
    std::vector<int64_t> ap(ni + 1, 0);
    std::vector<int32_t> ai;
    std::vector<double> ax;
    ai.reserve(adji.size() / 2 + ni);
    ax.reserve(adji.size() / 2 + ni);
    {
        std::vector<std::pair<int32_t, double>> rowbuf;
        for (int64_t k = 0; k < ni; ++k) {
            rowbuf.clear();
            const int32_t r = interior[order[k]];
            for (int64_t q = krowptr[r]; q < krowptr[r + 1]; ++q) {
                const int32_t j = iidx[kcol[q]];
                if (j < 0) continue;
                const int32_t pj = pos[j];
                // exact zeros (e.g. the diagonal edges of P1 on right triangles) are left out
                // here as in the dissection graph: the factor's pattern must be the graph's
                if (pj <= k && (kval[q] != 0.0 || pj == k)) rowbuf.emplace_back(pj, kval[q]);
            }
            std::sort(rowbuf.begin(), rowbuf.end());
            for (auto& e : rowbuf) {
                if (!ai.empty() && (int64_t)ai.size() > ap[k] && ai.back() == e.first) {
                    ax.back() += e.second;
                } else {
                    ai.push_back(e.first);
                    ax.push_back(e.second);
                }
            }
            ap[k + 1] = (int64_t)ai.size();
        }
    }
    // ---- elimination tree (Liu, with path compression)
    std::vector<int32_t> parent(ni, -1), anc(ni, -1);
    for (int64_t k = 0; k < ni; ++k) {
        for (int64_t q = ap[k]; q < ap[k + 1]; ++q) {
            int32_t j = ai[q];
            while (j != -1 && j < k) {
                const int32_t nxt = anc[j];
                anc[j] = (int32_t)k;
                if (nxt == -1) {
                    parent[j] = (int32_t)k;
                    break;
                }
                j = nxt;
            }
        }
    }
    // ---- row patterns by tree reach: column counts, then the numeric factorisation
    std::vector<int32_t> mark(ni, -1), stack;
    std::vector<int32_t> pat;
    auto reach = [&](int64_t k) {
        pat.clear();
        mark[k] = (int32_t)k;
        for (int64_t q = ap[k]; q < ap[k + 1]; ++q) {
            int32_t j = ai[q];
            while (j != -1 && j < k && mark[j] != k) {
                mark[j] = (int32_t)k;
                pat.push_back(j);
                j = parent[j];
            }
        }
        std::sort(pat.begin(), pat.end());
    };
    std::vector<int64_t> Lp(ni + 1, 0);
    for (int64_t k = 0; k < ni; ++k) {
        reach(k);
        for (int32_t j : pat) Lp[j + 1]++;
        Lp[k + 1]++;  // diagonal
    }
    for (int64_t k = 0; k < ni; ++k) Lp[k + 1] += Lp[k];
    const int64_t nnzL = Lp[ni];
    if (nnzL > (int64_t)INT32_MAX - 1) {
        f.err = "mean Cholesky: factor too large";
        return SGFEM_ERR_UNSUPPORTED;
    }
    std::vector<int32_t> Li(nnzL);
    std::vector<double> Lx(nnzL);
    std::vector<int64_t> next(Lp.begin(), Lp.end() - 1);
    std::fill(mark.begin(), mark.end(), -1);
    std::vector<double> x(ni, 0.0);
    for (int64_t k = 0; k < ni; ++k) {
        reach(k);
        double d = 0.0;
        for (int64_t q = ap[k]; q < ap[k + 1]; ++q) {
            if (ai[q] == k) d += ax[q];
            else x[ai[q]] = ax[q];
        }
        for (int32_t j : pat) {
            const double lkj = x[j] / Lx[Lp[j]];
            x[j] = 0.0;
            for (int64_t q = Lp[j] + 1; q < next[j]; ++q) x[Li[q]] -= Lx[q] * lkj;
            d -= lkj * lkj;
            Li[next[j]] = (int32_t)k;
            Lx[next[j]] = lkj;
            next[j]++;
        }
        if (!(d > 0.0)) {
            f.err = "mean Cholesky: K_0 is not positive definite on the interior dofs";
            return SGFEM_ERR_ARGUMENT;
        }
        Li[Lp[k]] = (int32_t)k;
        Lx[Lp[k]] = std::sqrt(d);
        next[k] = Lp[k] + 1;
    }
    // ---- per node: dense inverse of the diagonal block; gather lists
    std::vector<long long> off_of_node(nodes.size(), 0);
    size_t dtotal = 0;
    for (size_t id = 0; id < nodes.size(); ++id) {
        off_of_node[id] = (long long)dtotal;
        const size_t s = (size_t)(nodes[id].r1 - nodes[id].r0);
        dtotal += s * s;
    }
    if (dtotal > ((size_t)1 << 31)) {
        f.err = "mean Cholesky: separators too large";
        return SGFEM_ERR_UNSUPPORTED;
    }
    std::vector<double> dinv(dtotal, 0.0), dinvt(dtotal, 0.0);
    // backward gather = entries L(i, k) with i outside k's node (below it): the columns of L
    std::vector<int> bptr(ni + 1, 0), bcol;
    std::vector<double> bval;
    // forward gather = entries L(k, j) with j before k's node: rows of L (transpose of the columns)
    std::vector<int> fcount(ni + 1, 0);
    for (int64_t j = 0; j < ni; ++j) {
        const int nb1 = nodes[node_of[j]].r1;
        for (int64_t q = Lp[j] + 1; q < Lp[j + 1]; ++q) {
            const int32_t i = Li[q];
            if (i >= nb1) {
                bcol.push_back(i);
                bval.push_back(Lx[q]);
                fcount[i + 1]++;
            }
        }
        bptr[j + 1] = (int)bcol.size();
    }
    std::vector<int> fptr(ni + 1, 0);
    for (int64_t k = 0; k < ni; ++k) fptr[k + 1] = fptr[k] + fcount[k + 1];
    std::vector<int> fcol(fptr[ni]);
    std::vector<double> fval(fptr[ni]);
    {
        std::vector<int> fill(fptr.begin(), fptr.end() - 1);
        for (int64_t j = 0; j < ni; ++j)  // ascending j: each row's columns come out sorted
            for (int p = bptr[j]; p < bptr[j + 1]; ++p) {
                const int i = bcol[p];
                fcol[fill[i]] = (int)j;
                fval[fill[i]] = bval[p];
                fill[i]++;
            }
    }
    std::vector<double> blk;
    for (size_t id = 0; id < nodes.size(); ++id) {
        const int a = nodes[id].r0, s = nodes[id].r1 - nodes[id].r0;
        if (s == 0) continue;
        blk.assign((size_t)s * s, 0.0);  // L_KK row-major
        for (int jj = 0; jj < s; ++jj) {
            const int64_t j = a + jj;
            for (int64_t q = Lp[j]; q < Lp[j + 1]; ++q) {
                const int i = Li[q];
                if (i < a + s) blk[(size_t)(i - a) * s + jj] = Lx[q];
            }
        }
        // inverse of a lower-triangular block, column by column (forward substitution on e_c)
        double* D = dinv.data() + off_of_node[id];
        for (int c = 0; c < s; ++c) {
            for (int r = c; r < s; ++r) {
                double v = (r == c) ? 1.0 : 0.0;
                for (int u = c; u < r; ++u) v -= blk[(size_t)r * s + u] * D[(size_t)u * s + c];
                D[(size_t)r * s + c] = v / blk[(size_t)r * s + r];
            }
        }
        double* Dt = dinvt.data() + off_of_node[id];
        for (int r = 0; r < s; ++r)
            for (int c = 0; c < s; ++c) Dt[(size_t)c * s + r] = D[(size_t)r * s + c];
    }
    // ---- the schedule's premise: every gathered entry of a row lies in a strictly lower
    // node (forward) / strictly higher node (backward) of the dissection tree
    for (int64_t k = 0; k < ni; ++k)
        for (int p = fptr[k]; p < fptr[k + 1]; ++p)
            if (nodes[node_of[fcol[p]]].height >= nodes[node_of[k]].height) {
                f.err = "mean Cholesky: an entry of L couples two nodes that are not in descent";
                return SGFEM_ERR_UNSUPPORTED;
            }
    // ---- schedule by height
    int H = 0;
    for (auto& nd_ : nodes) H = std::max(H, nd_.height + 1);
    std::vector<int>& hptr = f.hptr;
    hptr.assign(H + 1, 0);
    for (int64_t e = 0; e < ni; ++e) hptr[nodes[node_of[e]].height + 1]++;
    for (int h = 0; h < H; ++h) hptr[h + 1] += hptr[h];
    std::vector<int> rows(ni);
    {
        std::vector<int> fill(hptr.begin(), hptr.end() - 1);
        for (int64_t e = 0; e < ni; ++e) rows[fill[nodes[node_of[e]].height]++] = (int)e;
    }
    std::vector<int> na(ni), ns(ni), dev(ni);
    std::vector<long long> noff(ni);
    for (int64_t e = 0; e < ni; ++e) {
        const NDNode& nd_ = nodes[node_of[e]];
        na[e] = nd_.r0;
        ns[e] = nd_.r1 - nd_.r0;
        noff[e] = off_of_node[node_of[e]];
        dev[e] = interior[order[e]];
    }
    std::vector<int> brows;
    for (int64_t i = 0; i < n; ++i)
        if (bmask[i]) brows.push_back((int)i);
    int maxs = 0;
    for (auto& nd_ : nodes) maxs = std::max(maxs, nd_.r1 - nd_.r0);
    f.dev = std::move(dev); f.rows = std::move(rows); f.na = std::move(na); f.ns = std::move(ns);
    f.noff = std::move(noff); f.fptr = std::move(fptr); f.fcol = std::move(fcol); f.fval = std::move(fval);
    f.bptr = std::move(bptr); f.bcol = std::move(bcol); f.bval = std::move(bval); f.dinv = std::move(dinv);
    f.dinvt = std::move(dinvt); f.brows = std::move(brows);
    f.nnzL = nnzL;
    f.nnodes = (int)nodes.size();
    f.H = H;
    f.maxs = maxs;
    return SGFEM_OK;
}

// The device schedule on the host, same order of every sum: Z = K_0^-1 R on the
// interior rows (R, Z: n x ld row-major in device numbering), boundary rows zero.
void host_solve(const HostFactor& f, int64_t n, int ld, const double* R, double* Z) {
    const int64_t ni = f.ni;
    std::vector<double> t((size_t)ni * ld), y((size_t)ni * ld);
    for (int b : f.brows)
        for (int c = 0; c < ld; ++c) Z[(size_t)b * ld + c] = 0.0;
    for (int h = 0; h < f.H; ++h) {
        for (int q = f.hptr[h]; q < f.hptr[h + 1]; ++q) {
            const int k = f.rows[q];
            for (int c = 0; c < ld; ++c) {
                double acc = R[(size_t)f.dev[k] * ld + c];
                for (int p = f.fptr[k]; p < f.fptr[k + 1]; ++p) acc -= f.fval[p] * y[(size_t)f.fcol[p] * ld + c];
                t[(size_t)k * ld + c] = acc;
            }
        }
        for (int q = f.hptr[h]; q < f.hptr[h + 1]; ++q) {
            const int k = f.rows[q], a = f.na[k], s = f.ns[k], r = k - a;
            const double* drow = f.dinv.data() + f.noff[k] + (size_t)r * s;
            for (int c = 0; c < ld; ++c) {
                double acc = 0.0;
                for (int u = 0; u <= r; ++u) acc += drow[u] * t[(size_t)(a + u) * ld + c];
                y[(size_t)k * ld + c] = acc;
            }
        }
    }
    for (int h = f.H - 1; h >= 0; --h) {
        for (int q = f.hptr[h]; q < f.hptr[h + 1]; ++q) {
            const int k = f.rows[q];
            for (int c = 0; c < ld; ++c) {
                double acc = y[(size_t)k * ld + c];
                for (int p = f.bptr[k]; p < f.bptr[k + 1]; ++p) acc -= f.bval[p] * y[(size_t)f.bcol[p] * ld + c];
                t[(size_t)k * ld + c] = acc;
            }
        }
        for (int q = f.hptr[h]; q < f.hptr[h + 1]; ++q) {
            const int k = f.rows[q], a = f.na[k], s = f.ns[k], r = k - a;
            const double* drow = f.dinvt.data() + f.noff[k] + (size_t)r * s;
            for (int c = 0; c < ld; ++c) {
                double acc = 0.0;
                for (int u = r; u < s; ++u) acc += drow[u] * t[(size_t)(a + u) * ld + c];
                y[(size_t)k * ld + c] = acc;
                Z[(size_t)f.dev[k] * ld + c] = acc;
            }
        }
    }
    (void)n;
}

int factor(sgfem_context* ctx, MeanChol* mc) {
    HostFactor f;
    const int st = host_factor(ctx->n, mc->rowptr, mc->col, mc->val, mc->interior, ctx->bmask_host, f);
    if (st != SGFEM_OK) return sg_fail(ctx, st, f.err);
    mc->ni = f.ni;
    mc->hptr = f.hptr;
    SG_TRY(upload_vec(ctx, &mc->d_dev, f.dev));
    SG_TRY(upload_vec(ctx, &mc->d_rows, f.rows));
    SG_TRY(upload_vec(ctx, &mc->d_na, f.na));
    SG_TRY(upload_vec(ctx, &mc->d_ns, f.ns));
    SG_TRY(upload_vec(ctx, &mc->d_noff, f.noff));
    SG_TRY(upload_vec(ctx, &mc->d_fptr, f.fptr));
    SG_TRY(upload_vec(ctx, &mc->d_fcol, f.fcol));
    SG_TRY(upload_vec(ctx, &mc->d_fval64, f.fval));
    SG_TRY(upload_vec(ctx, &mc->d_fval32, to_f32(f.fval)));
    SG_TRY(upload_vec(ctx, &mc->d_bptr, f.bptr));
    SG_TRY(upload_vec(ctx, &mc->d_bcol, f.bcol));
    SG_TRY(upload_vec(ctx, &mc->d_bval64, f.bval));
    SG_TRY(upload_vec(ctx, &mc->d_bval32, to_f32(f.bval)));
    SG_TRY(upload_vec(ctx, &mc->d_dinv64, f.dinv));
    SG_TRY(upload_vec(ctx, &mc->d_dinv32, to_f32(f.dinv)));
    SG_TRY(upload_vec(ctx, &mc->d_dinvt64, f.dinvt));
    SG_TRY(upload_vec(ctx, &mc->d_dinvt32, to_f32(f.dinvt)));
    SG_TRY(upload_vec(ctx, &mc->d_brows, f.brows));
    mc->nb = (int)f.brows.size();
    mc->nnzL = f.nnzL;
    mc->dinv_entries = f.dinv.size();
    mc->nnodes = f.nnodes;
    mc->log = "exact K_0^-1 by sparse Cholesky (nested dissection: " + std::to_string(f.nnodes) + " nodes, " +
              std::to_string(f.H) + " heights, largest node " + std::to_string(f.maxs) + " rows; nnz(L) " +
              std::to_string(f.nnzL) + ")";
    // host copies of K_0 are no longer needed
    mc->rowptr.clear(); mc->rowptr.shrink_to_fit();
    mc->col.clear(); mc->col.shrink_to_fit();
    mc->val.clear(); mc->val.shrink_to_fit();
    return SGFEM_OK;
}

template <typename T>
int apply_t(sgfem_context* ctx, MeanChol* mc, const T* R, T* Z, const KrylovScalars* scal) {
    const int ld = (int)ctx->ld;
    const int nchunk = (ld + 31) / 32;
    const int H = (int)mc->hptr.size() - 1;
    T* tt = (T*)mc->w_t.p;
    T* yy = (T*)mc->w_y.p;
    const bool f64 = sizeof(T) == 8;
    const T* fval = f64 ? (const T*)mc->d_fval64 : (const T*)mc->d_fval32;
    const T* bval = f64 ? (const T*)mc->d_bval64 : (const T*)mc->d_bval32;
    const T* dinv = f64 ? (const T*)mc->d_dinv64 : (const T*)mc->d_dinv32;
    const T* dinvt = f64 ? (const T*)mc->d_dinvt64 : (const T*)mc->d_dinvt32;
    if (mc->nb > 0) {
        const int g = (int)std::min<int64_t>(((int64_t)mc->nb * ld + 255) / 256, (int64_t)ctx->num_sms * 4);
        k_zero_rows<T><<<std::max(1, g), 256, 0, ctx->stream>>>(Z, mc->d_brows, mc->nb, ld, scal);
        SG_LAUNCHED(ctx);
    }
    for (int h = 0; h < H; ++h) {  // L y = R
        const int nr = mc->hptr[h + 1] - mc->hptr[h];
        if (nr == 0) continue;
        const int g = (nr * nchunk + kWarps - 1) / kWarps;
        const int* rows = mc->d_rows + mc->hptr[h];
        k_chol_gather<T><<<g, kWarps * 32, 0, ctx->stream>>>(rows, nr, nchunk, ld, mc->d_fptr, mc->d_fcol, fval, R,
                                                             mc->d_dev, yy, tt, scal);
        SG_LAUNCHED(ctx);
        k_chol_dense<T, false><<<g, kWarps * 32, 0, ctx->stream>>>(rows, nr, nchunk, ld, mc->d_na, mc->d_ns,
                                                                   mc->d_noff, dinv, tt, yy, nullptr, nullptr, scal);
        SG_LAUNCHED(ctx);
    }
    for (int h = H - 1; h >= 0; --h) {  // L^T z = y (z overwrites y node by node)
        const int nr = mc->hptr[h + 1] - mc->hptr[h];
        if (nr == 0) continue;
        const int g = (nr * nchunk + kWarps - 1) / kWarps;
        const int* rows = mc->d_rows + mc->hptr[h];
        k_chol_gather<T><<<g, kWarps * 32, 0, ctx->stream>>>(rows, nr, nchunk, ld, mc->d_bptr, mc->d_bcol, bval,
                                                             nullptr, nullptr, yy, tt, scal);
        SG_LAUNCHED(ctx);
        k_chol_dense<T, true><<<g, kWarps * 32, 0, ctx->stream>>>(rows, nr, nchunk, ld, mc->d_na, mc->d_ns,
                                                                  mc->d_noff, dinvt, tt, yy, mc->d_dev, Z, scal);
        SG_LAUNCHED(ctx);
    }
    return SGFEM_OK;
}

}  // namespace

int sg_chol_prepare(sgfem_context* ctx, const std::vector<int64_t>& rowptr, const std::vector<int32_t>& col,
                    const std::vector<double>& val64) {
    sg_chol_release(ctx);
    MeanChol* mc = new MeanChol();
    ctx->chol = mc;
    const int64_t n = ctx->n;
    const int M1 = ctx->M1;
    mc->rowptr.assign(n + 1, 0);
    for (int64_t i = 0; i < n; ++i) {
        if (!ctx->bmask_host[i]) {
            mc->interior.push_back((int32_t)i);
            for (int64_t k = rowptr[i]; k < rowptr[i + 1]; ++k) {
                mc->col.push_back(col[k]);
                mc->val.push_back(val64[(size_t)k * M1 + 0]);
            }
        }
        mc->rowptr[i + 1] = (int64_t)mc->col.size();
    }
    return SGFEM_OK;
}

int sg_chol_ensure(sgfem_context* ctx) {
    MeanChol* mc = ctx->chol;
    if (!mc) return sg_fail(ctx, SGFEM_ERR_STATE, "mean Cholesky: not prepared (context not finalized)");
    if (mc->factored) return mc->status == SGFEM_OK ? SGFEM_OK : sg_fail(ctx, mc->status, mc->log);
    SG_CUDA(ctx, cudaSetDevice(ctx->device));
    mc->factored = true;
    mc->status = factor(ctx, mc);
    if (mc->status != SGFEM_OK) {
        mc->log = "mean Cholesky failed: " + ctx->err;
        return mc->status;
    }
    return SGFEM_OK;
}

int sg_chol_workspace(sgfem_context* ctx, int precision) {
    MeanChol* mc = ctx->chol;
    const size_t bytes = std::max<size_t>(1, (size_t)mc->ni * ctx->ld * sg_elem_bytes(precision));
    SG_TRY(sg_ensure(ctx, mc->w_t, bytes));
    SG_TRY(sg_ensure(ctx, mc->w_y, bytes));
    return SGFEM_OK;
}

int sg_chol_apply(sgfem_context* ctx, int precision, const void* R, void* Z, const KrylovScalars* scal) {
    MeanChol* mc = ctx->chol;
    if (!mc || !mc->factored || mc->status != SGFEM_OK)
        return sg_fail(ctx, SGFEM_ERR_STATE, "mean Cholesky: factor missing");
    if (precision == SGFEM_FP64) return apply_t<double>(ctx, mc, (const double*)R, (double*)Z, scal);
    return apply_t<float>(ctx, mc, (const float*)R, (float*)Z, scal);
}

int sg_chol_finish(sgfem_context* ctx, int precision, const void* R, const void* Z, void* P, int mode, double* rz,
                   int* nblocks, const KrylovScalars* scal) {
    const int threads = 256;
    int grid = (int)std::min<int64_t>(((int64_t)ctx->n * ctx->ld + threads - 1) / threads, (int64_t)ctx->num_sms * 8);
    if (grid < 1) grid = 1;
    if (nblocks) *nblocks = grid;
    if (precision == SGFEM_FP64)
        k_chol_finish<double><<<grid, threads, 0, ctx->stream>>>((const double*)R, (const double*)Z, (double*)P,
                                                                 ctx->d_bmask, (int)ctx->n, (int)ctx->ld, mode, rz,
                                                                 scal);
    else
        k_chol_finish<float><<<grid, threads, 0, ctx->stream>>>((const float*)R, (const float*)Z, (float*)P,
                                                                ctx->d_bmask, (int)ctx->n, (int)ctx->ld, mode, rz,
                                                                scal);
    SG_LAUNCHED(ctx);
    return SGFEM_OK;
}

const char* sg_chol_log(const sgfem_context* ctx) {
    return ctx->chol ? ctx->chol->log.c_str() : "unavailable (context not finalized)";
}

extern "C" const char* sgfem_cholesky_log(const sgfem_context* ctx) {
    if (!ctx) return "null context";
    return sg_chol_log(ctx);
}

void sg_chol_release(sgfem_context* ctx) {
    MeanChol* mc = ctx->chol;
    if (!mc) return;
    void* ptrs[] = {mc->d_dev,    mc->d_rows,   mc->d_na,      mc->d_ns,      mc->d_noff,   mc->d_fptr,
                    mc->d_fcol,   mc->d_fval64, mc->d_fval32,  mc->d_bptr,    mc->d_bcol,   mc->d_bval64,
                    mc->d_bval32, mc->d_dinv64, mc->d_dinv32,  mc->d_dinvt64, mc->d_dinvt32, mc->d_brows,
                    mc->w_t.p,    mc->w_y.p};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    delete mc;
    ctx->chol = nullptr;
}

// Host-only check of the factorisation and of the device schedule (no GPU): K_0 as
// 1-based CSC (the reference's SparseMatrixCSC), 1-based boundary dofs, B and Z
// column-major n x P (SGFEVector.entries); Z = K_0^-1 B on interior rows, zero on
// boundary rows, summed in the device kernels' order.
extern "C" int sgfem_cholesky_host_solve(int64_t n, const int64_t* colptr, const int64_t* rowval,
                                         const double* nzval, int64_t nb, const int64_t* bdofs, int64_t P,
                                         const double* B, double* Z, char* msg, int msglen) {
    auto fail = [&](int code, const std::string& m) {
        if (msg && msglen > 0) {
            std::strncpy(msg, m.c_str(), (size_t)msglen - 1);
            msg[msglen - 1] = 0;
        }
        return code;
    };
    if (n <= 0 || n > (int64_t)INT32_MAX || !colptr || !rowval || !nzval || P <= 0 || !B || !Z || nb < 0 ||
        (nb > 0 && !bdofs))
        return fail(SGFEM_ERR_ARGUMENT, "bad arguments");
    if (colptr[0] != 1) return fail(SGFEM_ERR_ARGUMENT, "colptr must be 1-based");
    std::vector<unsigned char> bmask(n, 0);
    for (int64_t k = 0; k < nb; ++k) {
        if (bdofs[k] < 1 || bdofs[k] > n) return fail(SGFEM_ERR_ARGUMENT, "boundary dof out of range");
        bmask[bdofs[k] - 1] = 1;
    }
    // rows of the (symmetric) K_0 = its columns
    std::vector<int64_t> rp(n + 1, 0);
    std::vector<int32_t> cl;
    std::vector<double> vl;
    std::vector<int32_t> interior;
    for (int64_t j = 0; j < n; ++j) {
        if (!bmask[j]) {
            interior.push_back((int32_t)j);
            for (int64_t k = colptr[j] - 1; k < colptr[j + 1] - 1; ++k) {
                const int64_t r = rowval[k] - 1;
                if (r < 0 || r >= n) return fail(SGFEM_ERR_ARGUMENT, "row index out of range");
                cl.push_back((int32_t)r);
                vl.push_back(nzval[k]);
            }
        }
        rp[j + 1] = (int64_t)cl.size();
    }
    HostFactor f;
    const int st = host_factor(n, rp, cl, vl, interior, bmask, f);
    if (st != SGFEM_OK) return fail(st, f.err);
    const int ld = (int)P;
    std::vector<double> R((size_t)n * ld), Zr((size_t)n * ld);
    for (int64_t m = 0; m < P; ++m)
        for (int64_t i = 0; i < n; ++i) R[(size_t)i * ld + m] = B[m * n + i];
    host_solve(f, n, ld, R.data(), Zr.data());
    for (int64_t m = 0; m < P; ++m)
        for (int64_t i = 0; i < n; ++i) Z[m * n + i] = Zr[(size_t)i * ld + m];
    return fail(SGFEM_OK, "exact K_0^-1 by sparse Cholesky: " + std::to_string(f.nnodes) + " nodes, " +
                              std::to_string(f.H) + " heights, largest node " + std::to_string(f.maxs) +
                              " rows, nnz(L) " + std::to_string(f.nnzL));
}
