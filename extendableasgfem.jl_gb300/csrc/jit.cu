// Specialised FP32 SG apply, compiled at finalize time with NVRTC for the
// coupling structure of the operator (the same operator as k_apply, see
// apply.cu; mul!(Ax, S, x), src/modelproblems/solvers_poisson_primal.jl:86-124).
//
// Schedule (one warp per row):
//   * lane L owns device columns c = 32 k + L (k < KG): for each nonzero (i, j)
//     it loads X[j, c] once into a register and duplicates it into a float2;
//   * the M+1 values of the nonzero are loaded once as float4 vectors with a
//     warp-uniform address and read as pairs (K_2p, K_2p+1);
//   * one packed FP32x2 FMA per slot (pair p, group k) accumulates
//     (acc(2p, c), acc(2p+1, c)) += (K_2p[i,j], K_2p+1[i,j]) * X[j, c];
//     slots exist only where group k holds a column coupled to pair p, and the
//     device column order (sg_mode_order) packs those columns into few groups;
//   * after the row: accumulators to shared memory, then
//     Y[i, c] = sum_e g_e acc[off_e] over the per-column combination list
//     (K_0 term with g = 1, then the G entries), Dirichlet rows zero,
//     p'Ap partial in FP64.
// The slot list is compile-time, so every accumulator, KLE value and X value
// is a register and no instruction needs a lane-dependent shared-memory index.
// NVRTC and the driver entry points are loaded at run time; when they are not
// available the generic kernel (apply.cu) stays in use.
#include <cuda.h>
#include <dlfcn.h>
#include <nvrtc.h>

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "sgfem_internal.h"

namespace {

constexpr int JWPB = 4;  // warps per block

struct Nvrtc {
    bool loaded = false;
    bool tried = false;
    std::string err;
    nvrtcResult (*create)(nvrtcProgram*, const char*, const char*, int, const char* const*, const char* const*) = nullptr;
    nvrtcResult (*compile)(nvrtcProgram, int, const char* const*) = nullptr;
    nvrtcResult (*log_size)(nvrtcProgram, size_t*) = nullptr;
    nvrtcResult (*log)(nvrtcProgram, char*) = nullptr;
    nvrtcResult (*cubin_size)(nvrtcProgram, size_t*) = nullptr;
    nvrtcResult (*cubin)(nvrtcProgram, char*) = nullptr;
    nvrtcResult (*destroy)(nvrtcProgram*) = nullptr;
};

struct Driver {
    bool loaded = false;
    bool tried = false;
    std::string err;
    CUresult (*module_load_data)(CUmodule*, const void*) = nullptr;
    CUresult (*module_get_function)(CUfunction*, CUmodule, const char*) = nullptr;
    CUresult (*module_unload)(CUmodule) = nullptr;
    CUresult (*func_set_attribute)(CUfunction, CUfunction_attribute, int) = nullptr;
    CUresult (*launch_kernel)(CUfunction, unsigned, unsigned, unsigned, unsigned, unsigned, unsigned, unsigned,
                              CUstream, void**, void**) = nullptr;
    CUresult (*occupancy)(int*, CUfunction, int, size_t) = nullptr;
};

Nvrtc g_nvrtc;
Driver g_drv;

template <typename F>
bool sym(void* h, const char* name, F& f) {
    f = reinterpret_cast<F>(dlsym(h, name));
    return f != nullptr;
}

bool load_nvrtc() {
    if (g_nvrtc.tried) return g_nvrtc.loaded;
    g_nvrtc.tried = true;
    const char* names[] = {"libnvrtc.so.13", "/usr/local/cuda/lib64/libnvrtc.so.13", "libnvrtc.so",
                           "/usr/local/cuda/lib64/libnvrtc.so"};
    void* h = nullptr;
    for (const char* nm : names)
        if ((h = dlopen(nm, RTLD_NOW | RTLD_LOCAL))) break;
    if (!h) {
        g_nvrtc.err = "libnvrtc not found";
        return false;
    }
    bool ok = sym(h, "nvrtcCreateProgram", g_nvrtc.create) && sym(h, "nvrtcCompileProgram", g_nvrtc.compile) &&
              sym(h, "nvrtcGetProgramLogSize", g_nvrtc.log_size) && sym(h, "nvrtcGetProgramLog", g_nvrtc.log) &&
              sym(h, "nvrtcGetCUBINSize", g_nvrtc.cubin_size) && sym(h, "nvrtcGetCUBIN", g_nvrtc.cubin) &&
              sym(h, "nvrtcDestroyProgram", g_nvrtc.destroy);
    if (!ok) g_nvrtc.err = "libnvrtc lacks an entry point";
    g_nvrtc.loaded = ok;
    return ok;
}

template <typename F>
bool entry(const char* name, F& f) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion(name, &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess || !p)
        return false;
    f = reinterpret_cast<F>(p);
    return true;
}

bool load_driver() {
    if (g_drv.tried) return g_drv.loaded;
    g_drv.tried = true;
    bool ok = entry("cuModuleLoadData", g_drv.module_load_data) &&
              entry("cuModuleGetFunction", g_drv.module_get_function) &&
              entry("cuModuleUnload", g_drv.module_unload) && entry("cuFuncSetAttribute", g_drv.func_set_attribute) &&
              entry("cuLaunchKernel", g_drv.launch_kernel) &&
              entry("cuOccupancyMaxActiveBlocksPerMultiprocessor", g_drv.occupancy);
    if (!ok) g_drv.err = "driver entry points unavailable";
    g_drv.loaded = ok;
    return ok;
}

// the packed-FMA slots of one nonzero: a_q += (c[pair].lo, c[pair].hi) * (x_k, x_k)
std::string slot_fmas(const sgfem_context* ctx, const char* ind) {
    std::string s;
    char buf[256];
    const int NS = (int)ctx->jit_slots.size();
    for (int q = 0; q < NS; ++q) {
        const int pr = ctx->jit_slots[q].first, k = ctx->jit_slots[q].second;
        const int v = pr / 2;
        const char* comp = (pr % 2 == 0) ? "x, c%d.y" : "z, c%d.w";
        char cpair[64];
        snprintf(cpair, sizeof(cpair), comp, v);
        snprintf(buf, sizeof(buf), "%sa%d = __ffma2_rn(make_float2(c%d.%s), w%d, a%d);\n", ind, q, v, cpair, k, q);
        s += buf;
    }
    return s;
}

// x<d>_k = X[col of nonzero t, 32k + lane] for t < cnt (t warp-uniform), else 0
std::string loadx(const sgfem_context* ctx, int d, const std::string& t, const char* ind) {
    const int LD = (int)ctx->ld, KG = (int)((ctx->P + 31) / 32);
    std::string s;
    char buf[256];
    snprintf(buf, sizeof(buf), "%s{\n%s    const int tt_ = %s;\n%s    const int jj_ = __shfl_sync(0xffffffffu, jl, tt_ < cnt ? tt_ : 0);\n"
                               "%s    const float* xr_ = X + (size_t)jj_ * LD + lane;\n",
             ind, ind, t.c_str(), ind, ind);
    s += buf;
    for (int k = 0; k < KG; ++k) {
        const int valid = LD - 32 * k;
        if (valid >= 32)
            snprintf(buf, sizeof(buf), "%s    x%d_%d = (tt_ < cnt) ? __ldg(xr_ + %d) : 0.f;\n", ind, d, k, 32 * k);
        else
            snprintf(buf, sizeof(buf), "%s    x%d_%d = (tt_ < cnt && lane < %d) ? __ldg(xr_ + %d) : 0.f;\n", ind, d, k,
                     valid, 32 * k);
        s += buf;
    }
    s += ind;
    s += "}\n";
    return s;
}

std::string generate_source(const sgfem_context* ctx) {
    const int LD = (int)ctx->ld, P = (int)ctx->P, M1P = ctx->M1P;
    const int KG = (int)((P + 31) / 32);
    const int NS = (int)ctx->jit_slots.size();
    const int pfd = std::max(1, ctx->jit_pfd);
    std::string s;
    char buf[512];
    snprintf(buf, sizeof(buf),
             "#define LD %d\n#define P %d\n#define KG %d\n#define M1P %d\n#define NS %d\n#define WPB %d\n"
             "#define RCHUNK %d\n#define PREFETCH %d\n#define T %d\n#define STAGE %d\n#define PFD %d\n#define MINB %d\n"
             "#define NBUF %d\n#define DIFF %d\n",
             LD, P, KG, M1P, NS, JWPB, ctx->jit_rchunk, ctx->jit_prefetch, ctx->jit_T, ctx->jit_stage, pfd,
             ctx->jit_minb, ctx->jit_nbuf, ctx->jit_diff);
    s += buf;
    s += R"(
#define NV4 (M1P / 4)                 /* float4 per nonzero */
#if STAGE
#define CBUF (32 * M1P)               /* floats per value buffer (32 nonzeros) */
#else
#define CBUF 0
#endif
#define WSMEM (NS * 64 + NBUF * CBUF + ((LD + 3) & ~3))   /* floats per warp */
struct Scal { double rho, pq, alpha, beta, rr, tol2; int done, status, iters, first; };

__device__ __forceinline__ void pf_l1(const void* p) { asm volatile("prefetch.global.L1 [%0];" ::"l"(p)); }

// X rows of a row (columns lane-parallel in jl), prefetched into L1
__device__ __forceinline__ void prefetch_x(const float* __restrict__ X, int jl, int cnt, int lane) {
    const int total = cnt * KG;
    for (int q0 = 0; q0 < total; q0 += 32) {
        const int q = min(q0 + lane, total - 1);
        const int t = q / KG, k = q - t * KG;
        const int j = __shfl_sync(0xffffffffu, jl, t);
        if (q0 + lane < total) pf_l1(X + (size_t)j * LD + 32 * k);
    }
}

// values of up to 32 nonzeros starting at nz (cnt of them) -> registers (lane-parallel float4)
#define LOAD_VALUES(pv, nz, cnt)                                                        \
    _Pragma("unroll") for (int i_ = 0; i_ < NV4; ++i_) {                                \
        const int q_ = lane + 32 * i_;                                                  \
        pv[i_] = (q_ < (cnt) * NV4) ? __ldg(reinterpret_cast<const float4*>(vals + (size_t)(nz) * M1P) + q_) \
                                    : make_float4(0.f, 0.f, 0.f, 0.f);                  \
    }
#define STORE_VALUES(dst, pv)                                                           \
    _Pragma("unroll") for (int i_ = 0; i_ < NV4; ++i_)                                  \
        reinterpret_cast<float4*>(dst)[lane + 32 * i_] = pv[i_];

#if MINB > 0
extern "C" __global__ void __launch_bounds__(WPB * 32, MINB)
#else
extern "C" __global__ void __launch_bounds__(WPB * 32)
#endif
sg_apply_jit(const int* __restrict__ rowptr, const int* __restrict__ col, const float* __restrict__ vals,
             const float* __restrict__ X, float* __restrict__ Y, int n, const unsigned char* __restrict__ bmask,
             const int2* __restrict__ jtab, double* __restrict__ partials, const Scal* __restrict__ scal,
             int* __restrict__ err) {
    if (scal && scal->done) return;
    extern __shared__ __align__(16) float smem[];
    __shared__ double red[WPB];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    int2* stab = reinterpret_cast<int2*>(smem);
    float* wb = smem + 2 * T * 32 + warp * WSMEM;
    float* sacc = wb;
    float* cbuf = wb + NS * 64;
    float* ybuf = cbuf + NBUF * CBUF;
    for (int i = threadIdx.x; i < T * 32; i += blockDim.x) stab[i] = __ldg(jtab + i);
    __syncthreads();
    double dot = 0.0;
    // rows in bands: warp w takes RCHUNK consecutive rows of each band of
    // nw * RCHUNK rows (X rows reused across consecutive rows and across warps)
    const int nw = gridDim.x * WPB, w = blockIdx.x * WPB + warp;
    const int stride = nw * RCHUNK;
#define NEXT_ROW(r) ((((r) + 1) % RCHUNK) ? ((r) + 1) : ((r) + 1 - RCHUNK + stride))
    int row = w * RCHUNK;
    int jn1 = 0, cn1 = 0, b = 0;
    float4 pv[NV4];
    if (row < n) {
        const int a = rowptr[row];
        cn1 = min(32, rowptr[row + 1] - a);
        jn1 = (lane < cn1) ? __ldg(col + a + lane) : 0;
#if STAGE
        LOAD_VALUES(pv, a, cn1);
        STORE_VALUES(cbuf, pv);
#endif
        if (PREFETCH) prefetch_x(X, jn1, cn1, lane);
        __syncwarp();
    }
    for (; row < n; row = NEXT_ROW(row)) {
        const int jcur = jn1, ccur = cn1;
        const int r1n = NEXT_ROW(row);
        if (r1n < n) {  // next row: columns and values (first 32 nonzeros) into registers
            const int a = __ldg(rowptr + r1n);
            cn1 = min(32, __ldg(rowptr + r1n + 1) - a);
            jn1 = (lane < cn1) ? __ldg(col + a + lane) : 0;
#if STAGE
            LOAD_VALUES(pv, a, cn1);
#else
            if (PREFETCH) {  // values of the row after next into L1
                const int r2n = NEXT_ROW(r1n);
                if (r2n < n) {
                    const char* v0 = reinterpret_cast<const char*>(vals + (size_t)__ldg(rowptr + r2n) * M1P);
                    const char* v1 = reinterpret_cast<const char*>(vals + (size_t)__ldg(rowptr + r2n + 1) * M1P);
                    for (const char* q = v0 + lane * 128; q < v1; q += 32 * 128) pf_l1(q);
                }
            }
#endif
        }
        float* yrow = Y + (size_t)row * LD;
        if (bmask[row]) {
            for (int c = lane; c < LD; c += 32) yrow[c] = 0.f;
        } else {
)";
    for (int q = 0; q < NS; ++q) {
        snprintf(buf, sizeof(buf), "            float2 a%d = make_float2(0.f, 0.f);\n", q);
        s += buf;
    }
    // difference form: with vanishing row sums K x = sum_j K_ij (x_j - x_i); the own
    // row's values are subtracted from every gathered row (no cancellation in FP32)
    for (int k = 0; k < KG; ++k) {
        const int valid = LD - 32 * k;
        if (valid >= 32)
            snprintf(buf, sizeof(buf), "            const float xi%d = DIFF ? __ldg(X + (size_t)row * LD + %d + lane) : 0.f;\n", k, 32 * k);
        else
            snprintf(buf, sizeof(buf), "            const float xi%d = (DIFF && lane < %d) ? __ldg(X + (size_t)row * LD + %d + lane) : 0.f;\n", k, valid, 32 * k);
        s += buf;
    }
    s += R"(            const int nz0 = rowptr[row], nz1 = rowptr[row + 1];
            if (PREFETCH && r1n < n) prefetch_x(X, jn1, cn1, lane);
            const float* cb = cbuf + b * CBUF;
            for (int base = nz0; base < nz1; base += 32) {
                const int cnt = min(32, nz1 - base);
                int jl = jcur;
                if (base != nz0) {  // rows longer than 32 nonzeros: later chunks load synchronously
                    jl = (lane < cnt) ? __ldg(col + base + lane) : 0;
#if STAGE
                    float4 lv[NV4];
                    __syncwarp();
                    LOAD_VALUES(lv, base, cnt);
                    STORE_VALUES(cbuf + b * CBUF, lv);
                    __syncwarp();
#endif
                }
#if PFD <= 1
#pragma unroll 2
                for (int t = 0; t < cnt; ++t) {
                const int j = __shfl_sync(0xffffffffu, jl, t);
#if STAGE
                const float4* cv = reinterpret_cast<const float4*>(cb + t * M1P);
#else
                const float4* cv = reinterpret_cast<const float4*>(vals + (size_t)(base + t) * M1P);
#endif
                const float* xr = X + (size_t)j * LD + lane;
)";
    for (int v = 0; v < M1P / 4; ++v) {
        snprintf(buf, sizeof(buf), "                const float4 c%d = STAGE ? cv[%d] : __ldg(cv + %d);\n", v, v, v);
        s += buf;
    }
    for (int k = 0; k < KG; ++k) {
        const int valid = LD - 32 * k;
        if (valid >= 32)
            snprintf(buf, sizeof(buf), "                const float u%d = __ldg(xr + %d) - xi%d;\n", k, 32 * k, k);
        else
            snprintf(buf, sizeof(buf), "                const float u%d = (lane < %d) ? __ldg(xr + %d) - xi%d : 0.f;\n",
                     k, valid, 32 * k, k);
        s += buf;
        snprintf(buf, sizeof(buf), "                const float2 w%d = make_float2(u%d, u%d);\n", k, k, k);
        s += buf;
    }
    s += slot_fmas(ctx, "                ");
    s += "                }\n";
    s += "#else\n";
    // X values of the next PFD nonzeros rotate through PFD register sets: the loads
    // for nonzero t + PFD are issued right after nonzero t's values are taken
    for (int d = 0; d < pfd; ++d)
        for (int k = 0; k < KG; ++k) {
            snprintf(buf, sizeof(buf), "                float x%d_%d;\n", d, k);
            s += buf;
        }
    for (int d = 0; d < pfd; ++d) s += loadx(ctx, d, std::to_string(d), "                ");
    s += "                for (int t0 = 0; t0 < cnt; t0 += PFD) {\n";
    for (int d = 0; d < pfd; ++d) {
        snprintf(buf, sizeof(buf), "                if (t0 + %d < cnt) {\n", d);
        s += buf;
        snprintf(buf, sizeof(buf),
                 "#if STAGE\n                    const float4* cv = reinterpret_cast<const float4*>(cb + (t0 + %d) * M1P);\n"
                 "#else\n                    const float4* cv = reinterpret_cast<const float4*>(vals + (size_t)(base + t0 + %d) * M1P);\n#endif\n",
                 d, d);
        s += buf;
        for (int v = 0; v < M1P / 4; ++v) {
            snprintf(buf, sizeof(buf), "                    const float4 c%d = STAGE ? cv[%d] : __ldg(cv + %d);\n", v, v, v);
            s += buf;
        }
        for (int k = 0; k < KG; ++k) {
            snprintf(buf, sizeof(buf), "                    const float2 w%d = make_float2(x%d_%d - xi%d, x%d_%d - xi%d);\n", k, d, k,
                     k, d, k, k);
            s += buf;
        }
        s += loadx(ctx, d, "t0 + " + std::to_string(d + pfd), "                    ");
        s += slot_fmas(ctx, "                    ");
        s += "                }\n";
    }
    s += "                }\n";
    s += "#endif\n";
    s += "            }\n";
    for (int q = 0; q < NS; ++q) {
        snprintf(buf, sizeof(buf), "            *reinterpret_cast<float2*>(sacc + %d + 2 * lane) = a%d;\n", q * 64, q);
        s += buf;
    }
    s += R"(            __syncwarp();
            // combination: lane schedule, T entries per lane, store Y[c] at each column's last entry
            float acc = 0.f;
#pragma unroll
            for (int i = 0; i < T; ++i) {
                const int2 e = stab[i * 32 + lane];
                acc = fmaf(__int_as_float(e.y), sacc[e.x & 0x1fff], acc);
                if (e.x >> 28) {
                    ybuf[(e.x >> 13) & 0x7fff] = acc;
                    acc = 0.f;
                }
            }
            __syncwarp();
            const float* xrow = X + (size_t)row * LD;
            float rowdot = 0.f;  // per-row products in FP32, rows summed in FP64
            for (int c = lane; c < LD; c += 32) {
                const float y = (c < P) ? ybuf[c] : 0.f;
                yrow[c] = y;
                if (partials) rowdot = fmaf(xrow[c], y, rowdot);
            }
            dot += (double)rowdot;
        }
#if STAGE
        if (r1n < n) {  // stage the next row's values
            __syncwarp();
            b = (NBUF == 2) ? (b ^ 1) : 0;  // one buffer: the row's reads are done (syncwarp above)
            STORE_VALUES(cbuf + b * CBUF, pv);
            __syncwarp();
        }
#endif
    }
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

// Variant with an asynchronous copy pipeline: every warp streams, for the
// nonzeros of its rows in order, the X row of the nonzero's column and the
// nonzero's KLE values into a ring of ADEPTH shared-memory slots (cp.async,
// one commit group per nonzero) and consumes nonzero t while the copies of
// t+1 .. t+ADEPTH-1 are in flight.  The bytes in flight per SM then come
// from shared memory instead of registers.  The producer keeps the row
// metadata (row pointers, the column indices of 32 nonzeros) of its current
// and next row in registers, loaded one row ahead.
std::string generate_source_async(const sgfem_context* ctx) {
    const int LD = (int)ctx->ld, P = (int)ctx->P, M1P = ctx->M1P;
    const int KG = (int)((P + 31) / 32);
    const int NS = (int)ctx->jit_slots.size();
    std::string s;
    char buf[512];
    snprintf(buf, sizeof(buf),
             "#define LD %d\n#define P %d\n#define KG %d\n#define M1P %d\n#define NS %d\n#define WPB %d\n"
             "#define RCHUNK %d\n#define T %d\n#define ADEPTH %d\n#define MINB %d\n",
             LD, P, KG, M1P, NS, JWPB, ctx->jit_rchunk, ctx->jit_T, ctx->jit_adepth, ctx->jit_minb);
    s += buf;
    s += R"(
#define SLOTF (LD + M1P)              /* floats per ring slot: X row, then the KLE values */
#define NCH (SLOTF / 4)               /* 16-byte chunks per slot */
#define WSMEM (ADEPTH * SLOTF + NS * 64 + LD)   /* floats per warp */
struct Scal { double rho, pq, alpha, beta, rr, tol2; int done, status, iters, first; };

__device__ __forceinline__ void cp16(float* dst, const float* src) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 16;" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_wait_depth() { asm volatile("cp.async.wait_group %0;" ::"n"(ADEPTH - 1) : "memory"); }
__device__ __forceinline__ void cp_wait_all() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }

#if MINB > 0
extern "C" __global__ void __launch_bounds__(WPB * 32, MINB)
#else
extern "C" __global__ void __launch_bounds__(WPB * 32)
#endif
sg_apply_jit(const int* __restrict__ rowptr, const int* __restrict__ col, const float* __restrict__ vals,
             const float* __restrict__ X, float* __restrict__ Y, int n, const unsigned char* __restrict__ bmask,
             const int2* __restrict__ jtab, double* __restrict__ partials, const Scal* __restrict__ scal,
             int* __restrict__ err) {
    if (scal && scal->done) return;
    extern __shared__ __align__(16) float smem[];
    __shared__ double red[WPB];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    int2* stab = reinterpret_cast<int2*>(smem);
    float* ring = smem + 2 * T * 32 + warp * WSMEM;
    float* sacc = ring + ADEPTH * SLOTF;
    float* ybuf = sacc + NS * 64;
    for (int i = threadIdx.x; i < T * 32; i += blockDim.x) stab[i] = __ldg(jtab + i);
    __syncthreads();
    double dot = 0.0;
    const int nw = gridDim.x * WPB, w = blockIdx.x * WPB + warp;
    const int stride = nw * RCHUNK;
#define NEXT_ROW(r) ((((r) + 1) % RCHUNK) ? ((r) + 1) : ((r) + 1 - RCHUNK + stride))
    // ---- producer: the row being copied (prow: nonzeros [pnz, pend), column indices of
    // [pbase, pbase + 32) lane-wise in pjl) and the next row's metadata (q*), loaded ahead
    int prow = w * RCHUNK, pnz = 0, pend = 0, pbase = 0, pjl = 0;
    int qrow = 0, qnz = 0, qend = 0, qjl = 0;
    // first producer row with nonzeros off the boundary
    while (prow < n && (bmask[prow] || rowptr[prow] == rowptr[prow + 1])) prow = NEXT_ROW(prow);
    if (prow < n) {
        pnz = pbase = rowptr[prow];
        pend = rowptr[prow + 1];
        pjl = (lane < pend - pbase) ? __ldg(col + pbase + lane) : 0;
    }
    // next producer row (skips boundary and empty rows)
#define FETCH_NEXT()                                                                     \
    {                                                                                    \
        qrow = (prow < n) ? NEXT_ROW(prow) : n;                                          \
        while (qrow < n && (bmask[qrow] || rowptr[qrow] == rowptr[qrow + 1])) qrow = NEXT_ROW(qrow); \
        if (qrow < n) {                                                                  \
            qnz = rowptr[qrow];                                                          \
            qend = rowptr[qrow + 1];                                                     \
            qjl = (lane < qend - qnz) ? __ldg(col + qnz + lane) : 0;                     \
        }                                                                                \
    }
    FETCH_NEXT();
    int sp = 0;  // next slot to fill
    // copy one nonzero into slot sp; one commit group per call (empty once the rows run out)
#define PRODUCE()                                                                        \
    {                                                                                    \
        if (prow < n) {                                                                  \
            if (pnz - pbase >= 32) {                                                     \
                pbase = pnz;                                                             \
                pjl = (lane < pend - pbase) ? __ldg(col + pbase + lane) : 0;             \
            }                                                                            \
            const int j_ = __shfl_sync(0xffffffffu, pjl, pnz - pbase);                   \
            float* dst_ = ring + sp * SLOTF;                                             \
            const float* sx_ = X + (size_t)j_ * LD;                                      \
            const float* sv_ = vals + (size_t)pnz * M1P;                                 \
            for (int q_ = lane; q_ < NCH; q_ += 32)                                      \
                cp16(dst_ + 4 * q_, q_ < LD / 4 ? sx_ + 4 * q_ : sv_ + 4 * (q_ - LD / 4)); \
            if (++pnz == pend) {                                                         \
                prow = qrow; pnz = pbase = qnz; pend = qend; pjl = qjl;                  \
                FETCH_NEXT();                                                            \
            }                                                                            \
        }                                                                                \
        cp_commit();                                                                     \
        sp = (sp + 1 == ADEPTH) ? 0 : sp + 1;                                            \
    }
    for (int i = 0; i < ADEPTH - 1; ++i) PRODUCE();
    int sc = 0;  // next slot to consume
    for (int row = w * RCHUNK; row < n; row = NEXT_ROW(row)) {
        float* yrow = Y + (size_t)row * LD;
        if (bmask[row]) {
            for (int c = lane; c < LD; c += 32) yrow[c] = 0.f;
            continue;
        }
        const int nz0 = rowptr[row], nz1 = rowptr[row + 1];
)";
    for (int q = 0; q < NS; ++q) {
        snprintf(buf, sizeof(buf), "        float2 a%d = make_float2(0.f, 0.f);\n", q);
        s += buf;
    }
    s += R"(        for (int t = nz0; t < nz1; ++t) {
            PRODUCE();
            cp_wait_depth();
            __syncwarp();
            const float* sl = ring + sc * SLOTF;
            const float4* cv = reinterpret_cast<const float4*>(sl + LD);
)";
    for (int v = 0; v < M1P / 4; ++v) {
        snprintf(buf, sizeof(buf), "            const float4 c%d = cv[%d];\n", v, v);
        s += buf;
    }
    for (int k = 0; k < KG; ++k) {
        const int valid = LD - 32 * k;
        if (valid >= 32)
            snprintf(buf, sizeof(buf), "            const float u%d = sl[%d + lane];\n", k, 32 * k);
        else
            snprintf(buf, sizeof(buf), "            const float u%d = (lane < %d) ? sl[%d + lane] : 0.f;\n", k, valid,
                     32 * k);
        s += buf;
        snprintf(buf, sizeof(buf), "            const float2 w%d = make_float2(u%d, u%d);\n", k, k, k);
        s += buf;
    }
    s += R"(            __syncwarp();  // every lane has read the slot before it is refilled
            sc = (sc + 1 == ADEPTH) ? 0 : sc + 1;
)";
    s += slot_fmas(ctx, "            ");
    s += "        }\n";
    for (int q = 0; q < NS; ++q) {
        snprintf(buf, sizeof(buf), "        *reinterpret_cast<float2*>(sacc + %d + 2 * lane) = a%d;\n", q * 64, q);
        s += buf;
    }
    s += R"(        __syncwarp();
        float acc = 0.f;
#pragma unroll
        for (int i = 0; i < T; ++i) {
            const int2 e = stab[i * 32 + lane];
            acc = fmaf(__int_as_float(e.y), sacc[e.x & 0x1fff], acc);
            if (e.x >> 28) {
                ybuf[(e.x >> 13) & 0x7fff] = acc;
                acc = 0.f;
            }
        }
        __syncwarp();
        const float* xrow = X + (size_t)row * LD;
        float rowdot = 0.f;
        for (int c = lane; c < LD; c += 32) {
            const float y = (c < P) ? ybuf[c] : 0.f;
            yrow[c] = y;
            if (partials) rowdot = fmaf(xrow[c], y, rowdot);
        }
        dot += (double)rowdot;
        __syncwarp();
    }
    cp_wait_all();
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

// Variant with bulk copies: one lane per warp moves each nonzero's X row
// (LD floats) and KLE values (M1P floats) into a ring of ADEPTH shared-memory
// slots with two cp.async.bulk copies that complete on the slot's mbarrier
// (expect-tx of the slot's bytes); the other lanes only consume.  Waits on a
// slot poll mbarrier.try_wait.parity at most WAIT_LIMIT times; on a timeout
// the kernel sets *err, waits (bounded) for the copies it has in flight and
// returns.
std::string generate_source_bulk(const sgfem_context* ctx) {
    const int LD = (int)ctx->ld, P = (int)ctx->P, M1P = ctx->M1P;
    const int KG = (int)((P + 31) / 32);
    const int NS = (int)ctx->jit_slots.size();
    std::string s;
    char buf[512];
    snprintf(buf, sizeof(buf),
             "#define LD %d\n#define P %d\n#define KG %d\n#define M1P %d\n#define NS %d\n#define WPB %d\n"
             "#define RCHUNK %d\n#define T %d\n#define ADEPTH %d\n#define MINB %d\n",
             LD, P, KG, M1P, NS, JWPB, ctx->jit_rchunk, ctx->jit_T, ctx->jit_adepth, ctx->jit_minb);
    s += buf;
    s += R"(
#define SLOTF (LD + M1P)                          /* floats per ring slot: X row, then the KLE values */
#define WSMEM (ADEPTH * SLOTF + NS * 64 + LD + 2 * ADEPTH)   /* floats per warp (+ ADEPTH mbarriers) */
#define WAIT_LIMIT (1 << 20)
struct Scal { double rho, pq, alpha, beta, rr, tol2; int done, status, iters, first; };

__device__ __forceinline__ unsigned sh_addr(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(unsigned bar) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar) : "memory");
}
__device__ __forceinline__ void mbar_expect(unsigned bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
__device__ __forceinline__ void bulk_copy(unsigned dst, const void* src, unsigned bytes, unsigned bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                 ::"r"(dst), "l"(src), "r"(bytes), "r"(bar) : "memory");
}
__device__ __forceinline__ unsigned mbar_try(unsigned bar, unsigned parity) {
    unsigned ok;
    asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n}"
                 : "=r"(ok) : "r"(bar), "r"(parity) : "memory");
    return ok;
}
// bounded wait; 0 on timeout
__device__ __forceinline__ int mbar_wait(unsigned bar, unsigned parity) {
    for (int i = 0; i < WAIT_LIMIT; ++i)
        if (mbar_try(bar, parity)) return 1;
    return 0;
}

#if MINB > 0
extern "C" __global__ void __launch_bounds__(WPB * 32, MINB)
#else
extern "C" __global__ void __launch_bounds__(WPB * 32)
#endif
sg_apply_jit(const int* __restrict__ rowptr, const int* __restrict__ col, const float* __restrict__ vals,
             const float* __restrict__ X, float* __restrict__ Y, int n, const unsigned char* __restrict__ bmask,
             const int2* __restrict__ jtab, double* __restrict__ partials, const Scal* __restrict__ scal,
             int* __restrict__ err) {
    if (scal && scal->done) return;
    extern __shared__ __align__(16) float smem[];
    __shared__ double red[WPB];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    int2* stab = reinterpret_cast<int2*>(smem);
    float* ring = smem + 2 * T * 32 + warp * WSMEM;
    float* sacc = ring + ADEPTH * SLOTF;
    float* ybuf = sacc + NS * 64;
    unsigned long long* bars = reinterpret_cast<unsigned long long*>(ybuf + LD);
    const unsigned ring_a = sh_addr(ring), bars_a = sh_addr(bars);
    for (int i = threadIdx.x; i < T * 32; i += blockDim.x) stab[i] = __ldg(jtab + i);
    if (lane == 0) {
        for (int k = 0; k < ADEPTH; ++k) mbar_init(bars_a + 8 * k);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    double dot = 0.0;
    const int nw = gridDim.x * WPB, w = blockIdx.x * WPB + warp;
    const int stride = nw * RCHUNK;
#define NEXT_ROW(r) ((((r) + 1) % RCHUNK) ? ((r) + 1) : ((r) + 1 - RCHUNK + stride))
    int prow = w * RCHUNK, pnz = 0, pend = 0, pbase = 0, pjl = 0;
    int qrow = 0, qnz = 0, qend = 0, qjl = 0;
    while (prow < n && (bmask[prow] || rowptr[prow] == rowptr[prow + 1])) prow = NEXT_ROW(prow);
    if (prow < n) {
        pnz = pbase = rowptr[prow];
        pend = rowptr[prow + 1];
        pjl = (lane < pend - pbase) ? __ldg(col + pbase + lane) : 0;
    }
#define FETCH_NEXT()                                                                     \
    {                                                                                    \
        qrow = (prow < n) ? NEXT_ROW(prow) : n;                                          \
        while (qrow < n && (bmask[qrow] || rowptr[qrow] == rowptr[qrow + 1])) qrow = NEXT_ROW(qrow); \
        if (qrow < n) {                                                                  \
            qnz = rowptr[qrow];                                                          \
            qend = rowptr[qrow + 1];                                                     \
            qjl = (lane < qend - qnz) ? __ldg(col + qnz + lane) : 0;                     \
        }                                                                                \
    }
    FETCH_NEXT();
    int sp = 0, sc = 0, inflight = 0;
    unsigned phase = 0;  // bit k: parity of slot k's next completion
    // one nonzero into slot sp (nothing once the rows run out)
#define PRODUCE()                                                                        \
    {                                                                                    \
        if (prow < n) {                                                                  \
            if (pnz - pbase >= 32) {                                                     \
                pbase = pnz;                                                             \
                pjl = (lane < pend - pbase) ? __ldg(col + pbase + lane) : 0;             \
            }                                                                            \
            const int j_ = __shfl_sync(0xffffffffu, pjl, pnz - pbase);                   \
            if (lane == 0) {                                                             \
                const unsigned bar_ = bars_a + 8 * sp;                                   \
                const unsigned dst_ = ring_a + 4 * SLOTF * sp;                           \
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");             \
                mbar_expect(bar_, 4 * SLOTF);                                            \
                bulk_copy(dst_, X + (size_t)j_ * LD, 4 * LD, bar_);                      \
                bulk_copy(dst_ + 4 * LD, vals + (size_t)pnz * M1P, 4 * M1P, bar_);       \
            }                                                                            \
            ++inflight;                                                                  \
            sp = (sp + 1 == ADEPTH) ? 0 : sp + 1;                                        \
            if (++pnz == pend) {                                                         \
                prow = qrow; pnz = pbase = qnz; pend = qend; pjl = qjl;                  \
                FETCH_NEXT();                                                            \
            }                                                                            \
        }                                                                                \
    }
    for (int i = 0; i < ADEPTH - 1; ++i) PRODUCE();
    bool failed = false;
    for (int row = w * RCHUNK; row < n && !failed; row = NEXT_ROW(row)) {
        float* yrow = Y + (size_t)row * LD;
        if (bmask[row]) {
            for (int c = lane; c < LD; c += 32) yrow[c] = 0.f;
            continue;
        }
        const int nz0 = rowptr[row], nz1 = rowptr[row + 1];
)";
    for (int q = 0; q < NS; ++q) {
        snprintf(buf, sizeof(buf), "        float2 a%d = make_float2(0.f, 0.f);\n", q);
        s += buf;
    }
    s += R"(        for (int t = nz0; t < nz1; ++t) {
            PRODUCE();
            if (!mbar_wait(bars_a + 8 * sc, (phase >> sc) & 1u)) {
                failed = true;
                break;
            }
            phase ^= 1u << sc;
            --inflight;
            const float* sl = ring + sc * SLOTF;
            const float4* cv = reinterpret_cast<const float4*>(sl + LD);
)";
    for (int v = 0; v < M1P / 4; ++v) {
        snprintf(buf, sizeof(buf), "            const float4 c%d = cv[%d];\n", v, v);
        s += buf;
    }
    for (int k = 0; k < KG; ++k) {
        const int valid = LD - 32 * k;
        if (valid >= 32)
            snprintf(buf, sizeof(buf), "            const float u%d = sl[%d + lane];\n", k, 32 * k);
        else
            snprintf(buf, sizeof(buf), "            const float u%d = (lane < %d) ? sl[%d + lane] : 0.f;\n", k, valid,
                     32 * k);
        s += buf;
        snprintf(buf, sizeof(buf), "            const float2 w%d = make_float2(u%d, u%d);\n", k, k, k);
        s += buf;
    }
    s += R"(            __syncwarp();  // every lane has read the slot before it is refilled
            sc = (sc + 1 == ADEPTH) ? 0 : sc + 1;
)";
    s += slot_fmas(ctx, "            ");
    s += "        }\n        if (failed) break;\n";
    for (int q = 0; q < NS; ++q) {
        snprintf(buf, sizeof(buf), "        *reinterpret_cast<float2*>(sacc + %d + 2 * lane) = a%d;\n", q * 64, q);
        s += buf;
    }
    s += R"(        __syncwarp();
        float acc = 0.f;
#pragma unroll
        for (int i = 0; i < T; ++i) {
            const int2 e = stab[i * 32 + lane];
            acc = fmaf(__int_as_float(e.y), sacc[e.x & 0x1fff], acc);
            if (e.x >> 28) {
                ybuf[(e.x >> 13) & 0x7fff] = acc;
                acc = 0.f;
            }
        }
        __syncwarp();
        const float* xrow = X + (size_t)row * LD;
        float rowdot = 0.f;
        for (int c = lane; c < LD; c += 32) {
            const float y = (c < P) ? ybuf[c] : 0.f;
            yrow[c] = y;
            if (partials) rowdot = fmaf(xrow[c], y, rowdot);
        }
        dot += (double)rowdot;
        __syncwarp();
    }
    if (failed) {
        if (lane == 0) atomicExch(err, 1);
        // copies still in flight land in this warp's ring: wait for them (bounded) before exiting
        for (int k = 0; k < inflight; ++k) {
            mbar_wait(bars_a + 8 * sc, (phase >> sc) & 1u);
            phase ^= 1u << sc;
            sc = (sc + 1 == ADEPTH) ? 0 : sc + 1;
        }
    }
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

// Variant with the column groups split into passes (jit_np > 1): for every row
// the warp runs over the row's nonzeros once per pass, loading only the pass's X
// column groups and keeping only the pass's slot accumulators, then folds the
// pass into ybuf with the pass's part of the combination schedule.  Fewer live
// accumulators and a smaller slot buffer per warp let more warps share an SM.
std::string generate_source_passes(const sgfem_context* ctx) {
    const int LD = (int)ctx->ld, P = (int)ctx->P, M1P = ctx->M1P;
    const int KG = (int)((P + 31) / 32);
    const int NP = ctx->jit_np;
    int maxps = 0;
    for (int p = 0; p < NP; ++p) maxps = std::max(maxps, ctx->jit_pass_slot0[p + 1] - ctx->jit_pass_slot0[p]);
    std::string s;
    char buf[512];
    snprintf(buf, sizeof(buf),
             "#define LD %d\n#define P %d\n#define KG %d\n#define M1P %d\n#define NSP %d\n#define WPB %d\n"
             "#define RCHUNK %d\n#define T %d\n#define MINB %d\n",
             LD, P, KG, M1P, maxps, JWPB, ctx->jit_rchunk, ctx->jit_T, ctx->jit_minb);
    s += buf;
    s += R"(
#define NV4 (M1P / 4)
#define CBUF (32 * M1P)
#define WSMEM (NSP * 64 + 2 * CBUF + LD)   /* floats per warp */
struct Scal { double rho, pq, alpha, beta, rr, tol2; int done, status, iters, first; };

#define LOAD_VALUES(pv, nz, cnt)                                                        \
    _Pragma("unroll") for (int i_ = 0; i_ < NV4; ++i_) {                                \
        const int q_ = lane + 32 * i_;                                                  \
        pv[i_] = (q_ < (cnt) * NV4) ? __ldg(reinterpret_cast<const float4*>(vals + (size_t)(nz) * M1P) + q_) \
                                    : make_float4(0.f, 0.f, 0.f, 0.f);                  \
    }
#define STORE_VALUES(dst, pv)                                                           \
    _Pragma("unroll") for (int i_ = 0; i_ < NV4; ++i_)                                  \
        reinterpret_cast<float4*>(dst)[lane + 32 * i_] = pv[i_];

#if MINB > 0
extern "C" __global__ void __launch_bounds__(WPB * 32, MINB)
#else
extern "C" __global__ void __launch_bounds__(WPB * 32)
#endif
sg_apply_jit(const int* __restrict__ rowptr, const int* __restrict__ col, const float* __restrict__ vals,
             const float* __restrict__ X, float* __restrict__ Y, int n, const unsigned char* __restrict__ bmask,
             const int2* __restrict__ jtab, double* __restrict__ partials, const Scal* __restrict__ scal,
             int* __restrict__ err) {
    if (scal && scal->done) return;
    extern __shared__ __align__(16) float smem[];
    __shared__ double red[WPB];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    int2* stab = reinterpret_cast<int2*>(smem);
    float* wb = smem + 2 * T * 32 + warp * WSMEM;
    float* sacc = wb;
    float* cbuf = wb + NSP * 64;
    float* ybuf = cbuf + 2 * CBUF;
    for (int i = threadIdx.x; i < T * 32; i += blockDim.x) stab[i] = __ldg(jtab + i);
    __syncthreads();
    double dot = 0.0;
    const int nw = gridDim.x * WPB, w = blockIdx.x * WPB + warp;
    const int stride = nw * RCHUNK;
#define NEXT_ROW(r) ((((r) + 1) % RCHUNK) ? ((r) + 1) : ((r) + 1 - RCHUNK + stride))
    int row = w * RCHUNK;
    int jn1 = 0, cn1 = 0, b = 0;
    float4 pv[NV4];
    if (row < n) {
        const int a = rowptr[row];
        cn1 = min(32, rowptr[row + 1] - a);
        jn1 = (lane < cn1) ? __ldg(col + a + lane) : 0;
        LOAD_VALUES(pv, a, cn1);
        STORE_VALUES(cbuf, pv);
        __syncwarp();
    }
    for (; row < n; row = NEXT_ROW(row)) {
        const int jcur = jn1;
        const int r1n = NEXT_ROW(row);
        if (r1n < n) {
            const int a = __ldg(rowptr + r1n);
            cn1 = min(32, __ldg(rowptr + r1n + 1) - a);
            jn1 = (lane < cn1) ? __ldg(col + a + lane) : 0;
            LOAD_VALUES(pv, a, cn1);
        }
        float* yrow = Y + (size_t)row * LD;
        if (bmask[row]) {
            for (int c = lane; c < LD; c += 32) yrow[c] = 0.f;
        } else {
            const int nz0 = rowptr[row], nz1 = rowptr[row + 1];
            for (int c = lane; c < LD; c += 32) ybuf[c] = 0.f;
            const float* cb = cbuf + b * CBUF;
)";
    int toff = 0;
    for (int p = 0; p < NP; ++p) {
        const int s0 = ctx->jit_pass_slot0[p], s1 = ctx->jit_pass_slot0[p + 1];
        const int k0 = ctx->jit_pass_k0[p], k1 = ctx->jit_pass_k0[p + 1];
        // KLE value float4s this pass reads
        std::vector<char> usev(M1P / 4, 0);
        for (int q = s0; q < s1; ++q) usev[ctx->jit_slots[q].first / 2] = 1;
        snprintf(buf, sizeof(buf), "            // ---- pass %d: column groups [%d, %d), slots [%d, %d)\n            {\n", p, k0,
                 k1, s0, s1);
        s += buf;
        for (int q = s0; q < s1; ++q) {
            snprintf(buf, sizeof(buf), "            float2 a%d = make_float2(0.f, 0.f);\n", q);
            s += buf;
        }
        s += R"(            for (int base = nz0; base < nz1; base += 32) {
                const int cnt = min(32, nz1 - base);
                int jl = jcur;
                if (base != nz0) {  // rows longer than 32 nonzeros: later chunks load synchronously
                    jl = (lane < cnt) ? __ldg(col + base + lane) : 0;
                    float4 lv[NV4];
                    __syncwarp();
                    LOAD_VALUES(lv, base, cnt);
                    STORE_VALUES(cbuf + b * CBUF, lv);
                    __syncwarp();
                }
#pragma unroll 2
                for (int t = 0; t < cnt; ++t) {
                const int j = __shfl_sync(0xffffffffu, jl, t);
                const float4* cv = reinterpret_cast<const float4*>(cb + t * M1P);
                const float* xr = X + (size_t)j * LD + lane;
)";
        for (int v = 0; v < M1P / 4; ++v)
            if (usev[v]) {
                snprintf(buf, sizeof(buf), "                const float4 c%d = cv[%d];\n", v, v);
                s += buf;
            }
        for (int k = k0; k < k1; ++k) {
            const int valid = LD - 32 * k;
            if (valid >= 32)
                snprintf(buf, sizeof(buf), "                const float u%d = __ldg(xr + %d);\n", k, 32 * k);
            else
                snprintf(buf, sizeof(buf), "                const float u%d = (lane < %d) ? __ldg(xr + %d) : 0.f;\n",
                         k, valid, 32 * k);
            s += buf;
            snprintf(buf, sizeof(buf), "                const float2 w%d = make_float2(u%d, u%d);\n", k, k, k);
            s += buf;
        }
        for (int q = s0; q < s1; ++q) {
            const int pr = ctx->jit_slots[q].first, k = ctx->jit_slots[q].second;
            const int v = pr / 2;
            const char* comp = (pr % 2 == 0) ? "x, c%d.y" : "z, c%d.w";
            char cpair[64];
            snprintf(cpair, sizeof(cpair), comp, v);
            snprintf(buf, sizeof(buf), "                a%d = __ffma2_rn(make_float2(c%d.%s), w%d, a%d);\n", q, v, cpair,
                     k, q);
            s += buf;
        }
        s += "                }\n            }\n";
        for (int q = s0; q < s1; ++q) {
            snprintf(buf, sizeof(buf), "            *reinterpret_cast<float2*>(sacc + %d + 2 * lane) = a%d;\n",
                     (q - s0) * 64, q);
            s += buf;
        }
        snprintf(buf, sizeof(buf), R"(            __syncwarp();
            {
                float acc = 0.f;
#pragma unroll
                for (int i = 0; i < %d; ++i) {
                    const int2 e = stab[(%d + i) * 32 + lane];
                    acc = fmaf(__int_as_float(e.y), sacc[e.x & 0x1fff], acc);
                    if (e.x >> 28) {
                        ybuf[(e.x >> 13) & 0x7fff] += acc;
                        acc = 0.f;
                    }
                }
            }
            __syncwarp();
            }
)",
                 ctx->jit_pass_T[p], toff);
        s += buf;
        toff += ctx->jit_pass_T[p];
    }
    s += R"(            const float* xrow = X + (size_t)row * LD;
            float rowdot = 0.f;
            for (int c = lane; c < LD; c += 32) {
                const float y = (c < P) ? ybuf[c] : 0.f;
                yrow[c] = y;
                if (partials) rowdot = fmaf(xrow[c], y, rowdot);
            }
            dot += (double)rowdot;
        }
        if (r1n < n) {  // stage the next row's values
            __syncwarp();
            b ^= 1;
            STORE_VALUES(cbuf + b * CBUF, pv);
            __syncwarp();
        }
    }
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

// Variant for operators whose rows are the points of a uniform dof lattice
// (row = y * NLX + x) with couplings inside |dx| <= HX, |dy| <= HY: the
// gathered X rows come from a shared-memory window instead of L2.  The
// lattice is cut into strips of W = WPB * RW columns; a persistent block
// walks up its share of (strip, line) steps and keeps the X rows of lines
// y - HY .. y + HY of its strip plus HX halo columns on each side in a ring
// of WL = 2 HY + 2 line slots (cp.async, 16-byte pieces).  Line y + HY + 1 is
// copied while line y is computed; one barrier per line.  Warp w computes the
// RW rows x0 + w RW + r of each line with the packed-FMA slots and the
// combination of the register-window kernel; KLE values are staged per warp
// one row ahead, in the storage that holds the accumulators during the
// combination.  A column outside the window (a pattern that breaks the bounds
// found at finalize) sets bit 4 of the status word and contributes nothing.
std::string generate_source_window(const sgfem_context* ctx) {
    const int LD = (int)ctx->ld, P = (int)ctx->P, M1P = ctx->M1P;
    const int KG = (int)((P + 31) / 32);
    const int NS = (int)ctx->jit_slots.size();
    std::string s;
    char buf[512];
    snprintf(buf, sizeof(buf),
             "#define LD %d\n#define P %d\n#define KG %d\n#define M1P %d\n#define NS %d\n#define WPB %d\n"
             "#define T %d\n#define DIFF %d\n#define NLX %d\n#define NLY %d\n#define HX %d\n#define HY %d\n#define RW %d\n",
             LD, P, KG, M1P, NS, ctx->jit_wwpb, ctx->jit_T, ctx->jit_diff, ctx->lat_np, ctx->lat_np, ctx->win_hx,
             ctx->win_hy, ctx->jit_wrw);
    s += buf;
    s += R"(
#define NV4 (M1P / 4)
#define W (WPB * RW)                  /* rows of a strip per line */
#define SW (W + 2 * HX)               /* window columns */
#define WL (2 * HY + 2)               /* window line slots */
#define NSTRIP ((NLX + W - 1) / W)
#define LINES (NSTRIP * NLY)          /* (strip, line) steps */
#define CBUF (32 * M1P)
#define AREG (NS * 64 > CBUF ? NS * 64 : CBUF)
#define WSMEM (AREG + ((LD + 3) & ~3))
#define WIN (WL * SW * LD)
struct Scal { double rho, pq, alpha, beta, rr, tol2; int done, status, iters, first; };

__device__ __forceinline__ void cp16(float* dst, const float* src) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_wait_all() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }

// lattice line ly, columns [max(0, xs), min(NLX, xs + SW)) -> its ring slot
__device__ __forceinline__ void copy_line(float* win, const float* __restrict__ X, int ly, int xs) {
    const int cx0 = max(0, xs), cx1 = min(NLX, xs + SW);
    const int n4 = (cx1 - cx0) * (LD / 4);
    const float* src = X + ((size_t)ly * NLX + cx0) * LD;
    float* dst = win + ((ly % WL) * SW + (cx0 - xs)) * LD;
    for (int i = threadIdx.x; i < n4; i += WPB * 32) cp16(dst + 4 * i, src + 4 * i);
}

#define LOAD_VALUES(pv, nz, cnt)                                                        \
    _Pragma("unroll") for (int i_ = 0; i_ < NV4; ++i_) {                                \
        const int q_ = lane + 32 * i_;                                                  \
        pv[i_] = (q_ < (cnt) * NV4) ? __ldg(reinterpret_cast<const float4*>(vals + (size_t)(nz) * M1P) + q_) \
                                    : make_float4(0.f, 0.f, 0.f, 0.f);                  \
    }
#define STORE_VALUES(dst, pv)                                                           \
    _Pragma("unroll") for (int i_ = 0; i_ < NV4; ++i_)                                  \
        reinterpret_cast<float4*>(dst)[lane + 32 * i_] = pv[i_];

// row of the warp's k-th step in a segment (k = (line - ya) * RW + r), -1 past the lattice edge
__device__ __forceinline__ int seg_row(int k, int ya, int x0, int warp) {
    const int x = x0 + warp * RW + k % RW;
    return x < NLX ? (ya + k / RW) * NLX + x : -1;
}

extern "C" __global__ void __launch_bounds__(WPB * 32, 1)
sg_apply_jit(const int* __restrict__ rowptr, const int* __restrict__ col, const float* __restrict__ vals,
             const float* __restrict__ X, float* __restrict__ Y, int n, const unsigned char* __restrict__ bmask,
             const int2* __restrict__ jtab, double* __restrict__ partials, const Scal* __restrict__ scal,
             int* __restrict__ err) {
    if (scal && scal->done) return;
    extern __shared__ __align__(16) float smem[];
    __shared__ double red[WPB];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    int2* stab = reinterpret_cast<int2*>(smem);
    float* win = smem + 2 * T * 32;
    float* wb = win + WIN + warp * WSMEM;
    float* sacc = wb;
    float* cbuf = wb;
    float* ybuf = wb + AREG;
    for (int i = threadIdx.x; i < T * 32; i += blockDim.x) stab[i] = __ldg(jtab + i);
    double dot = 0.0;
    int bad = 0;
    const int g0 = (int)(((long long)blockIdx.x * LINES) / gridDim.x);
    const int g1 = (int)(((long long)(blockIdx.x + 1) * LINES) / gridDim.x);
    for (int g = g0; g < g1;) {
        const int strip = g / NLY, ya = g - strip * NLY;
        const int yb = min(NLY, ya + (g1 - g));
        g += yb - ya;
        const int x0 = strip * W, xs = x0 - HX;
        __syncthreads();  // every read of the previous segment's window is done
        for (int ly = max(0, ya - HY); ly <= min(NLY - 1, ya + HY); ++ly) copy_line(win, X, ly, xs);
        cp_commit();
        const int KR = (yb - ya) * RW;
        // the warp's first row: its columns and values
        int k = 0;
        while (k < KR && seg_row(k, ya, x0, warp) < 0) ++k;
        int jn1 = 0, cn1 = 0;
        float4 pv[NV4];
        if (k < KR) {
            const int r0 = seg_row(k, ya, x0, warp);
            const int a = __ldg(rowptr + r0);
            cn1 = min(32, __ldg(rowptr + r0 + 1) - a);
            jn1 = (lane < cn1) ? __ldg(col + a + lane) : 0;
            LOAD_VALUES(pv, a, cn1);
            STORE_VALUES(cbuf, pv);
        }
        for (int kk = 0; kk < KR; ++kk) {
            if (kk % RW == 0) {  // new line: its window lines are present, start copying the next one
                const int y = ya + kk / RW;
                cp_wait_all();
                __syncthreads();
                if (y + HY + 1 < NLY && y + 1 < yb) copy_line(win, X, y + HY + 1, xs);
                cp_commit();
            }
            const int row = seg_row(kk, ya, x0, warp);
            if (row < 0) continue;  // warp-uniform: past the lattice edge
            const int y = ya + kk / RW, x = row - y * NLX;
            const int jcur = jn1, ccur = cn1;
            int kn = kk + 1;
            while (kn < KR && seg_row(kn, ya, x0, warp) < 0) ++kn;
            const int r1n = kn < KR ? seg_row(kn, ya, x0, warp) : -1;
            if (r1n >= 0) {  // next row: columns and values (first 32 nonzeros) into registers
                const int a = __ldg(rowptr + r1n);
                cn1 = min(32, __ldg(rowptr + r1n + 1) - a);
                jn1 = (lane < cn1) ? __ldg(col + a + lane) : 0;
                LOAD_VALUES(pv, a, cn1);
            }
            float* yrow = Y + (size_t)row * LD;
            const float* xown = win + ((y % WL) * SW + (x - xs)) * LD;
            if (bmask[row]) {
                for (int c = lane; c < LD; c += 32) yrow[c] = 0.f;
            } else {
)";
    for (int q = 0; q < NS; ++q) {
        snprintf(buf, sizeof(buf), "                float2 a%d = make_float2(0.f, 0.f);\n", q);
        s += buf;
    }
    for (int k = 0; k < KG; ++k) {
        const int valid = LD - 32 * k;
        if (valid >= 32)
            snprintf(buf, sizeof(buf), "                const float xi%d = DIFF ? xown[%d + lane] : 0.f;\n", k, 32 * k);
        else
            snprintf(buf, sizeof(buf), "                const float xi%d = (DIFF && lane < %d) ? xown[%d + lane] : 0.f;\n", k,
                     valid, 32 * k);
        s += buf;
    }
    s += R"(                const int nz0 = __ldg(rowptr + row), nz1 = __ldg(rowptr + row + 1);
                for (int base = nz0; base < nz1; base += 32) {
                    const int cnt = min(32, nz1 - base);
                    int jl = jcur;
                    if (base != nz0) {  // rows longer than 32 nonzeros: later chunks load synchronously
                        jl = (lane < cnt) ? __ldg(col + base + lane) : 0;
                        float4 lv[NV4];
                        __syncwarp();
                        LOAD_VALUES(lv, base, cnt);
                        STORE_VALUES(cbuf, lv);
                        __syncwarp();
                    } else {
                        (void)ccur;
                    }
                    // window offset of each lane's nonzero
                    int off = (int)(xown - win);
                    if (lane < cnt) {
                        const int cy = jl / NLX, cx = jl - cy * NLX;
                        const int dy = cy - y, wx = cx - xs;
                        if (dy < -HY || dy > HY || wx < 0 || wx >= SW) bad = 1;
                        else off = ((cy % WL) * SW + wx) * LD;
                    }
#pragma unroll UNROLL
                    for (int t = 0; t < cnt; ++t) {
                        const float* xr = win + __shfl_sync(0xffffffffu, off, t) + lane;
                        const float4* cv = reinterpret_cast<const float4*>(cbuf + t * M1P);
)";
    for (int v = 0; v < M1P / 4; ++v) {
        snprintf(buf, sizeof(buf), "                        const float4 c%d = cv[%d];\n", v, v);
        s += buf;
    }
    for (int k = 0; k < KG; ++k) {
        const int valid = LD - 32 * k;
        if (valid >= 32)
            snprintf(buf, sizeof(buf), "                        const float u%d = xr[%d] - xi%d;\n", k, 32 * k, k);
        else
            snprintf(buf, sizeof(buf), "                        const float u%d = (lane < %d) ? xr[%d] - xi%d : 0.f;\n", k,
                     valid, 32 * k, k);
        s += buf;
        snprintf(buf, sizeof(buf), "                        const float2 w%d = make_float2(u%d, u%d);\n", k, k, k);
        s += buf;
    }
    s += slot_fmas(ctx, "                        ");
    s += "                    }\n";
    s += "                }\n";
    s += "                __syncwarp();  // staged values read: their storage takes the accumulators\n";
    for (int q = 0; q < NS; ++q) {
        snprintf(buf, sizeof(buf), "                *reinterpret_cast<float2*>(sacc + %d + 2 * lane) = a%d;\n", q * 64, q);
        s += buf;
    }
    s += R"(                __syncwarp();
                float acc = 0.f;
#pragma unroll
                for (int i = 0; i < T; ++i) {
                    const int2 e = stab[i * 32 + lane];
                    acc = fmaf(__int_as_float(e.y), sacc[e.x & 0x1fff], acc);
                    if (e.x >> 28) {
                        ybuf[(e.x >> 13) & 0x7fff] = acc;
                        acc = 0.f;
                    }
                }
                __syncwarp();
                float rowdot = 0.f;
                for (int c = lane; c < LD; c += 32) {
                    const float yv = (c < P) ? ybuf[c] : 0.f;
                    yrow[c] = yv;
                    if (partials) rowdot = fmaf(xown[c], yv, rowdot);
                }
                dot += (double)rowdot;
            }
            if (r1n >= 0) {  // stage the next row's values (accumulator reads are done)
                __syncwarp();
                STORE_VALUES(cbuf, pv);
                __syncwarp();
            }
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
    const std::string pu = "#pragma unroll UNROLL";
    const size_t at = s.find(pu);
    if (at != std::string::npos) s.replace(at, pu.size(), "#pragma unroll " + std::to_string(ctx->jit_unroll));
    return s;
}

size_t window_smem_bytes(const sgfem_context* ctx, int wpb) {
    const size_t NS = ctx->jit_slots.size();
    const size_t W = (size_t)wpb * ctx->jit_wrw, SW = W + 2 * (size_t)ctx->win_hx, WL = 2 * (size_t)ctx->win_hy + 2;
    const size_t areg = std::max(NS * 64, (size_t)32 * ctx->M1P);
    const size_t wsmem = areg + ((ctx->ld + 3) & ~(size_t)3);
    return (2 * (size_t)ctx->jit_T * 32 + WL * SW * ctx->ld + wpb * wsmem) * sizeof(float);
}

size_t jit_smem_bytes(const sgfem_context* ctx) {
    if (ctx->jit_split) return sg_split_smem(ctx, ctx->jit_wwpb);
    const int NS = (int)ctx->jit_slots.size();
    if (ctx->jit_window) return window_smem_bytes(ctx, ctx->jit_wwpb);
    if (ctx->jit_np > 1 && !ctx->jit_async) {
        int maxps = 0;
        for (int p = 0; p < ctx->jit_np; ++p)
            maxps = std::max(maxps, ctx->jit_pass_slot0[p + 1] - ctx->jit_pass_slot0[p]);
        const size_t wsmem = (size_t)maxps * 64 + 2 * 32 * (size_t)ctx->M1P + ctx->ld;
        return (2 * (size_t)ctx->jit_T * 32 + JWPB * wsmem) * sizeof(float);
    }
    if (ctx->jit_async) {
        const size_t wsmem = (size_t)ctx->jit_adepth * (ctx->ld + ctx->M1P) + (size_t)NS * 64 + ctx->ld +
                             (ctx->jit_async == 2 ? 2 * (size_t)ctx->jit_adepth : 0);
        return (2 * (size_t)ctx->jit_T * 32 + JWPB * wsmem) * sizeof(float);
    }
    const size_t wsmem = (size_t)NS * 64 + (ctx->jit_stage ? (size_t)ctx->jit_nbuf * 32 * ctx->M1P : 0) + ((ctx->ld + 3) & ~3);
    return (2 * (size_t)ctx->jit_T * 32 + JWPB * wsmem) * sizeof(float);
}

}  // namespace

// knobs are read when the context is finalized (the kernel itself is compiled later)
void sg_jit_configure(sgfem_context* ctx) {
    const char* env = getenv("SGFEM_APPLY");
    ctx->jit_disabled = env && std::string(env) == "generic";
    const char* er = getenv("SGFEM_JIT_RCHUNK");
    const char* ep = getenv("SGFEM_JIT_PREFETCH");
    ctx->jit_rchunk = er ? std::max(1, atoi(er)) : 2;
    ctx->jit_prefetch = ep ? (atoi(ep) != 0) : 0;
    const char* es = getenv("SGFEM_JIT_STAGE");
    const char* eb = getenv("SGFEM_JIT_BPS");
    const char* ec = getenv("SGFEM_JIT_CARVEOUT");
    ctx->jit_stage = es ? (atoi(es) != 0) : 1;
    ctx->jit_bps_cap = eb ? std::max(1, atoi(eb)) : 8;
    ctx->jit_carveout = ec ? atoi(ec) : -1;
    const char* ed = getenv("SGFEM_JIT_PFD");
    ctx->jit_pfd = ed ? std::max(1, std::min(8, atoi(ed))) : 1;
    const char* ea = getenv("SGFEM_JIT_ASYNC");
    ctx->jit_async = ea ? std::max(0, std::min(2, atoi(ea))) : 0;
    const char* eq = getenv("SGFEM_JIT_ADEPTH");
    ctx->jit_adepth = eq ? std::max(2, std::min(16, atoi(eq))) : 6;
    const char* eb2 = getenv("SGFEM_JIT_NBUF");
    ctx->jit_nbuf = eb2 ? std::max(1, std::min(2, atoi(eb2))) : 1;
    const char* ewn = getenv("SGFEM_JIT_WINDOW");
    ctx->jit_window_req = ewn ? (atoi(ewn) != 0) : 1;
    const char* eww = getenv("SGFEM_JIT_WWPB");
    ctx->jit_wwpb = eww ? std::max(1, std::min(32, atoi(eww))) : 12;
    const char* ewr = getenv("SGFEM_JIT_WRW");
    ctx->jit_wrw = ewr ? std::max(1, std::min(8, atoi(ewr))) : 2;
    const char* eun = getenv("SGFEM_JIT_UNROLL");
    ctx->jit_unroll = eun ? std::max(1, std::min(4, atoi(eun))) : 1;
    const char* edf = getenv("SGFEM_JIT_DIFF");
    ctx->jit_diff_req = edf ? (atoi(edf) != 0) : 1;
    const char* en = getenv("SGFEM_JIT_PASSES");
    ctx->jit_np_req = en ? std::max(1, std::min(8, atoi(en))) : 1;
    if (ctx->jit_async) ctx->jit_np_req = 1;  // the copy-pipeline variants use one pass
    const char* esp = getenv("SGFEM_JIT_SPLIT");
    ctx->jit_split_req = esp ? (atoi(esp) != 0) : 0;  // measured slower than the pair-slot form
    const char* em = getenv("SGFEM_JIT_MINB");
    ctx->jit_minb = em ? std::max(0, std::min(8, atoi(em))) : 0;
}

int sg_jit_build(sgfem_context* ctx) {
    ctx->jit_ok = false;
    // lattice-window kernel: lattice-ordered rows with short couplings, one pass, and a
    // window that fits shared memory with at least 4 warps per block
    ctx->jit_window = 0;
    ctx->jit_split = 0;
    std::string split_why;
    if (ctx->jit_window_req && ctx->lat_order && !ctx->jit_async && ctx->jit_np <= 1 && ctx->win_hx <= 4 &&
        ctx->win_hy <= 4 && ctx->ld % 4 == 0 && ctx->jit_T > 0) {
        // split-slot form first (jit_split.cu), else the pair-slot window form
        if (ctx->jit_split_req && sg_split_plan(ctx, split_why) == SGFEM_OK) {
            if (sg_split_upload(ctx) != SGFEM_OK) split_why = "split tables: device allocation failed";
            // block shape of the split form: 16 warps of one row per lattice line unless asked otherwise
            if (!getenv("SGFEM_JIT_WWPB")) ctx->jit_wwpb = 16;
            if (!getenv("SGFEM_JIT_WRW")) ctx->jit_wrw = 1;
            int wpb = ctx->jit_wwpb;
            while (wpb >= 4 && sg_split_smem(ctx, wpb) > 220 * 1024) --wpb;
            if (!split_why.empty()) {
                sg_split_release(ctx);
            } else if (wpb >= 4) {
                ctx->jit_wwpb = wpb;
                ctx->jit_window = 1;
                ctx->jit_split = 1;
            } else {
                sg_split_release(ctx);
                split_why = "window does not fit shared memory";
            }
        }
        if (!ctx->jit_split) {
            if (!getenv("SGFEM_JIT_WWPB")) ctx->jit_wwpb = 12;
            if (!getenv("SGFEM_JIT_WRW")) ctx->jit_wrw = 2;
            int wpb = ctx->jit_wwpb;
            while (wpb >= 4 && window_smem_bytes(ctx, wpb) > 220 * 1024) --wpb;
            if (wpb >= 4) {
                ctx->jit_wwpb = wpb;
                ctx->jit_window = 1;
            }
        }
    }
    // the difference form is generated by the single-pass kernels only
    ctx->jit_diff = (ctx->jit_diff_req && ctx->rowsum_zero && !ctx->jit_async && ctx->jit_np <= 1) ? 1 : 0;
    if (ctx->jit_disabled) {
        ctx->jit_log = "disabled by SGFEM_APPLY=generic";
        return SGFEM_ERR_UNSUPPORTED;
    }
    const int NS = (int)ctx->jit_slots.size();
    if (NS == 0 || NS > 96 || ctx->M1P > 64 || ctx->jit_T <= 0 || ctx->jit_T > 256) {
        ctx->jit_log = "slot count outside the specialised kernel's range";
        return SGFEM_ERR_UNSUPPORTED;
    }
    if (!load_nvrtc()) {
        ctx->jit_log = g_nvrtc.err;
        return SGFEM_ERR_UNSUPPORTED;
    }
    if (!load_driver()) {
        ctx->jit_log = g_drv.err;
        return SGFEM_ERR_UNSUPPORTED;
    }
    const std::string src = ctx->jit_split ? sg_split_source(ctx)
                            : ctx->jit_window ? generate_source_window(ctx)
                            : ctx->jit_async == 2 ? generate_source_bulk(ctx)
                            : ctx->jit_async ? generate_source_async(ctx)
                            : ctx->jit_np > 1 ? generate_source_passes(ctx) : generate_source(ctx);
    nvrtcProgram prog = nullptr;
    if (g_nvrtc.create(&prog, src.c_str(), "sgfem_apply_jit.cu", 0, nullptr, nullptr) != NVRTC_SUCCESS) {
        ctx->jit_log = "nvrtcCreateProgram failed";
        return SGFEM_ERR_UNSUPPORTED;
    }
    const char* opts[] = {"--gpu-architecture=sm_103a", "--std=c++17", "-default-device", "-lineinfo"};
    nvrtcResult rc = g_nvrtc.compile(prog, 4, opts);
    size_t ls = 0;
    g_nvrtc.log_size(prog, &ls);
    std::string log(ls, '\0');
    if (ls) g_nvrtc.log(prog, &log[0]);
    if (rc != NVRTC_SUCCESS) {
        ctx->jit_log = "NVRTC compile failed: " + log;
        g_nvrtc.destroy(&prog);
        return SGFEM_ERR_UNSUPPORTED;
    }
    size_t cs = 0;
    g_nvrtc.cubin_size(prog, &cs);
    std::vector<char> cubin(cs);
    g_nvrtc.cubin(prog, cubin.data());
    g_nvrtc.destroy(&prog);
    CUmodule mod = nullptr;
    CUfunction fn = nullptr;
    if (g_drv.module_load_data(&mod, cubin.data()) != CUDA_SUCCESS) {
        ctx->jit_log = "cuModuleLoadData failed";
        return SGFEM_ERR_UNSUPPORTED;
    }
    if (g_drv.module_get_function(&fn, mod, "sg_apply_jit") != CUDA_SUCCESS) {
        g_drv.module_unload(mod);
        ctx->jit_log = "cuModuleGetFunction failed";
        return SGFEM_ERR_UNSUPPORTED;
    }
    const int smem = (int)jit_smem_bytes(ctx);
    if (smem > 220 * 1024) {
        g_drv.module_unload(mod);
        ctx->jit_log = "specialised apply needs too much shared memory";
        return SGFEM_ERR_UNSUPPORTED;
    }
    if (smem > 48 * 1024 &&
        g_drv.func_set_attribute(fn, CU_FUNC_ATTRIBUTE_MAX_DYNAMIC_SHARED_SIZE_BYTES, smem) != CUDA_SUCCESS) {
        g_drv.module_unload(mod);
        ctx->jit_log = "cuFuncSetAttribute failed";
        return SGFEM_ERR_UNSUPPORTED;
    }
    if (ctx->jit_carveout >= 0)
        g_drv.func_set_attribute(fn, CU_FUNC_ATTRIBUTE_PREFERRED_SHARED_MEMORY_CARVEOUT, ctx->jit_carveout);
    int bps = 0;
    if (g_drv.occupancy(&bps, fn, (ctx->jit_window ? ctx->jit_wwpb : JWPB) * 32, (size_t)smem) != CUDA_SUCCESS ||
        bps < 1) {
        g_drv.module_unload(mod);
        ctx->jit_log = "occupancy query failed";
        return SGFEM_ERR_UNSUPPORTED;
    }
    if (!ctx->d_jit_err) {
        if (cudaMalloc((void**)&ctx->d_jit_err, sizeof(int)) != cudaSuccess ||
            cudaMemset(ctx->d_jit_err, 0, sizeof(int)) != cudaSuccess) {
            g_drv.module_unload(mod);
            ctx->d_jit_err = nullptr;
            ctx->jit_log = "status word allocation failed";
            return SGFEM_ERR_UNSUPPORTED;
        }
    }
    ctx->jit_blocks_per_sm = std::min(bps, ctx->jit_bps_cap);
    ctx->jit_module = mod;
    ctx->jit_func = fn;
    ctx->jit_ok = true;
    ctx->jit_log = "specialised FP32 apply: " + std::to_string(NS) + " slots, " + std::to_string(bps) +
                   " blocks/SM, rows/chunk " + std::to_string(ctx->jit_rchunk) + ", prefetch " +
                   std::to_string(ctx->jit_prefetch) + ", staged values " + std::to_string(ctx->jit_stage) +
                   (ctx->jit_diff ? ", difference form" : "") +
                   (ctx->jit_window ? ", lattice window " + std::to_string(ctx->jit_wwpb * ctx->jit_wrw) + " x " +
                                          std::to_string(2 * ctx->win_hy + 2) + " lines, " +
                                          std::to_string(ctx->jit_wwpb) + " warps"
                                    : std::string()) +
                   (ctx->jit_split ? ", " + sg_split_summary(ctx)
                                   : (split_why.empty() ? std::string() : " (split form not used: " + split_why + ")"));
    return SGFEM_OK;
}

bool sg_jit_accepts(const sgfem_context* ctx, const void* X) {
    return ctx->jit_ok && (!ctx->jit_window || ((uintptr_t)X % 16) == 0);
}

int sg_jit_grid(const sgfem_context* ctx) {
    if (ctx->jit_window) {
        const int64_t W = (int64_t)ctx->jit_wwpb * ctx->jit_wrw;
        const int64_t lines = (ctx->lat_np + W - 1) / W * ctx->lat_np;
        return (int)std::max<int64_t>(1, std::min<int64_t>(lines, (int64_t)ctx->num_sms * std::min(ctx->jit_blocks_per_sm, 8)));
    }
    // persistent: one wave of resident blocks, each warp a contiguous row range
    const int64_t want = (ctx->n + JWPB - 1) / JWPB;
    const int64_t resident = (int64_t)ctx->num_sms * std::min(ctx->jit_blocks_per_sm, 8);
    return (int)std::max<int64_t>(1, std::min<int64_t>(want, resident));
}

int sg_jit_launch(sgfem_context* ctx, const void* X, void* Y, double* partials, int grid, const KrylovScalars* scal) {
    const unsigned smem = (unsigned)jit_smem_bytes(ctx);
    const int* rowptr = ctx->d_rowptr;
    const int* colp = ctx->d_col;
    const float* vals = ctx->d_val32p;
    int n = (int)ctx->n;
    const unsigned char* bm = ctx->d_bmask;
    const int2* jtab = ctx->d_jtab;
    int* errp = ctx->d_jit_err;
    void* args[] = {(void*)&rowptr, (void*)&colp, (void*)&vals, (void*)&X, (void*)&Y, (void*)&n, (void*)&bm,
                    (void*)&jtab, (void*)&partials, (void*)&scal, (void*)&errp};
    const int2* sjtab = nullptr;
    const int* lanetab = nullptr;
    void* sargs[] = {(void*)&rowptr, (void*)&colp, (void*)&vals, (void*)&X, (void*)&Y, (void*)&n, (void*)&bm,
                     (void*)&sjtab, (void*)&lanetab, (void*)&partials, (void*)&scal, (void*)&errp};
    if (ctx->jit_split) {
        sjtab = sg_split_jtab(ctx);
        lanetab = sg_split_lanetab(ctx);
    }
    const unsigned threads = (unsigned)(ctx->jit_window ? ctx->jit_wwpb : JWPB) * 32;
    CUresult r = g_drv.launch_kernel((CUfunction)ctx->jit_func, grid, 1, 1, threads, 1, 1, smem,
                                     (CUstream)ctx->stream, ctx->jit_split ? sargs : args, nullptr);
    if (r != CUDA_SUCCESS) return sg_fail(ctx, SGFEM_ERR_CUDA, "cuLaunchKernel(sg_apply_jit) failed: " + std::to_string((int)r));
    ctx->launches++;
    return SGFEM_OK;
}

// status word of the specialised kernel (a timed-out copy wait); resets it
int sg_jit_check(sgfem_context* ctx) {
    if (!ctx->jit_ok || !ctx->d_jit_err) return SGFEM_OK;
    int h = 0;
    SG_CUDA(ctx, cudaMemcpyAsync(&h, ctx->d_jit_err, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    SG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (h == 0) return SGFEM_OK;
    SG_CUDA(ctx, cudaMemsetAsync(ctx->d_jit_err, 0, sizeof(int), ctx->stream));
    if (h & 4) return sg_fail(ctx, SGFEM_ERR_CUDA, "specialised apply: a column outside the lattice window");
    return sg_fail(ctx, SGFEM_ERR_CUDA, "specialised apply: a shared-memory copy did not complete in time");
}

void sg_jit_release(sgfem_context* ctx) {
    sg_split_release(ctx);
    ctx->jit_split = 0;
    if (ctx->d_jit_err) cudaFree(ctx->d_jit_err);
    ctx->d_jit_err = nullptr;
    if (ctx->jit_module && g_drv.loaded) g_drv.module_unload((CUmodule)ctx->jit_module);
    ctx->jit_module = nullptr;
    ctx->jit_func = nullptr;
    ctx->jit_ok = false;
}

int sg_jit_ensure(sgfem_context* ctx) {
    if (ctx->jit_tried || ctx->batched || !ctx->finalized) return SGFEM_OK;
    ctx->jit_tried = true;
    if (sg_jit_build(ctx) != SGFEM_OK) ctx->err.clear();  // the generic kernel stays in use
    return SGFEM_OK;
}

// queries compile the specialised kernel if that has not happened yet
extern "C" int sgfem_apply_variant(const sgfem_context* ctx) {
    if (!ctx) return 0;
    if (ctx->finalized && !ctx->jit_tried && cudaSetDevice(ctx->device) == cudaSuccess)
        sg_jit_ensure(const_cast<sgfem_context*>(ctx));
    return ctx->jit_ok ? 1 : 0;
}

extern "C" const char* sgfem_apply_variant_log(const sgfem_context* ctx) {
    if (!ctx) return "null context";
    sgfem_apply_variant(ctx);
    return ctx->jit_log.c_str();
}
