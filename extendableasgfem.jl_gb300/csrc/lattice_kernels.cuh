// Device code of the lattice preconditioner (the transforms and pass kernels of
// lattice.cu), included by lattice.cu (FP32 instantiations and the host side) and
// lattice_f64.cu (FP64 instantiations), so that the two compile in parallel.  The
// kernels live in each unit's anonymous namespace; the geometry and the kernel
// pointer types are shared (namespace sglat).
#pragma once

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <type_traits>
#include <vector>

#include "sgfem_internal.h"

namespace sglat {

struct LatGeom {
    int Nl;     // transform length n = Nl (power of two), interior points N = Nl - 1
    int lg;     // log2(Nl)
    int ld;     // row stride of SG vectors
    int nchunk; // ceil(ld / 32)
    int async;  // the loaded vector is 16-byte aligned: lines are copied with cp.async
};

template <typename T>
using PassXFn = void (*)(const T*, T*, const T*, LatGeom, int, const KrylovScalars*);
template <typename T>
using PassYFn = void (*)(T*, const T*, const T*, LatGeom, double*, const KrylovScalars*);

// the FP64 kernel tables (lattice_f64.cu), L = Nl/2 = 2^LGL complex points, LGL = 1..8
PassXFn<double> pass_x_fn_f64(int LGL);
PassYFn<double> pass_y_fn_f64(int LGL);
PassYFn<double> pass_yb_fn_f64(int LGL);

}  // namespace sglat

namespace {

using sglat::LatGeom;

constexpr int LAT_THREADS = 256;
constexpr bool kLatScalarFFT = false;  // true: the scalar FFT for FP32 lines too
constexpr int LAT_WARPS = LAT_THREADS / 32;



// table layout (length 3*Nl/2 + 1):
//   [0, Nl/2)          cos(2 pi k / Nl)
//   [Nl/2, Nl)         sin(2 pi k / Nl)
//   [Nl, 3Nl/2 + 1)    sin(pi j / Nl), j = 0..Nl/2
// cos(pi m / 8), m = 0..8: the roots of unity of order 16 used inside a group
__device__ __forceinline__ constexpr double cos_pi8(int m) {
    return m == 0 ? 1.0
         : m == 1 ? 0.92387953251128675613
         : m == 2 ? 0.70710678118654752440
         : m == 3 ? 0.38268343236508977173
         : m == 4 ? 0.0
         : m == 5 ? -0.38268343236508977173
         : m == 6 ? -0.70710678118654752440
         : m == 7 ? -0.92387953251128675613
                  : -1.0;
}

// Radix-2 DIF FFT of the L = 2^LGL complex slots of every line of the tile,
// sign +.  Stages are done in chunks of up to 4 bits: each thread loads the
// 16 points of one group (indices differing only in the chunk's bits) into
// registers, runs the chunk's stages there and writes back, so a 256-point
// transform takes two shared-memory round trips instead of eight.  The
// twiddle of stage b (span h = 2^b) at t = bl + k' 2^lo (bl = the group's bits
// below the chunk, k' = the point's chunk bits below b) factors as
//   exp(i pi t / h) = omega^(2^(hi-b)) * exp(i pi k' / 2^(b-lo)),
// omega = exp(i pi bl / 2^hi) read once per group (and squared from stage to
// stage), the second factor a compile-time root of unity of order <= 16.
template <typename T, int LGL>
__device__ __forceinline__ void fft_dif(T* tile, const T* cs, const T* sn, int lane, int warp) {
    constexpr int L = 1 << LGL;
    constexpr int RB = LGL < 4 ? LGL : 4;
    // the last chunk (lo = 0) keeps all of a thread's groups in registers and stores
    // them to their bit-reversed slots, so the output is in natural order
    constexpr int NBL = (LGL - 1) % RB + 1;
    constexpr int NGW = ((L >> NBL) + LAT_WARPS - 1) / LAT_WARPS;
    T rel[NGW][1 << RB], iml[NGW][1 << RB];
#pragma unroll
    for (int hi = LGL - 1; hi >= 0; hi -= RB) {
        const int lo = hi - RB + 1 > 0 ? hi - RB + 1 : 0;
        const int nb = hi - lo + 1;
        const int G = 1 << nb;
        const int ngroups = L >> nb;
#pragma unroll
        for (int w = 0; w < (lo == 0 ? NGW : (L >> nb) / LAT_WARPS + 1); ++w) {
            const int g = warp + w * LAT_WARPS;
            if (g >= ngroups) break;
            const int base = ((g >> lo) << (hi + 1)) | (g & ((1 << lo) - 1));
            T* re = rel[lo == 0 ? w : 0];
            T* im = iml[lo == 0 ? w : 0];
#pragma unroll
            for (int k = 0; k < (1 << RB); ++k)
                if (k < G) {
                    const int idx = base | (k << lo);
                    re[k] = tile[(2 * idx) * 32 + lane];
                    im[k] = tile[(2 * idx + 1) * 32 + lane];
                }
            T omr = T(1), omi = T(0);
            if (lo > 0) {
                const int j = (g & ((1 << lo) - 1)) << (LGL - hi);
                omr = cs[j];
                omi = sn[j];
            }
#pragma unroll
            for (int bb = RB - 1; bb >= 0; --bb) {
                if (bb >= nb) continue;
                if (bb != nb - 1) {  // omega^(2^(hi-b)) from the previous stage's power
                    const T sr = omr * omr - omi * omi, si = T(2) * omr * omi;
                    omr = sr;
                    omi = si;
                }
                const int hs = 1 << bb;
#pragma unroll
                for (int k = 0; k < (1 << RB); ++k)
                    if (k < G && !(k & hs)) {
                        const int k2 = k | hs;
                        const T ar = re[k], ai = im[k], cr = re[k2], ci = im[k2];
                        re[k] = ar + cr;
                        im[k] = ai + ci;
                        const T dr = ar - cr, di = ai - ci;
                        const int m = (k & (hs - 1)) << (3 - bb);  // compile-time after unrolling
                        T wr = omr, wi = omi;
                        if (m != 0) {
                            const T c = (T)cos_pi8(m), sgn = (T)cos_pi8(m > 4 ? m - 4 : 4 - m);
                            wr = omr * c - omi * sgn;
                            wi = omr * sgn + omi * c;
                        }
                        re[k2] = dr * wr - di * wi;
                        im[k2] = dr * wi + di * wr;
                    }
            }
            if (lo != 0) {
#pragma unroll
                for (int k = 0; k < (1 << RB); ++k)
                    if (k < G) {
                        const int idx = base | (k << lo);
                        tile[(2 * idx) * 32 + lane] = re[k];
                        tile[(2 * idx + 1) * 32 + lane] = im[k];
                    }
            }
        }
        if (lo == 0) {
            __syncthreads();  // every input of the last chunk is in registers
#pragma unroll
            for (int w = 0; w < NGW; ++w) {
                const int g = warp + w * LAT_WARPS;
                if (g >= ngroups) break;
#pragma unroll
                for (int k = 0; k < (1 << RB); ++k)
                    if (k < G) {
                        const int idx = g * G + k;
                        const int r = (int)(__brev((unsigned)idx) >> (32 - LGL));
                        tile[(2 * r) * 32 + lane] = rel[w][k];
                        tile[(2 * r + 1) * 32 + lane] = iml[w][k];
                    }
            }
        }
        __syncthreads();
    }
}

// The same transform for FP32 lines whose length is a power of 16 (4-bit chunks
// only), with packed FP32x2 arithmetic: a group's 16 points are held as 8
// register pairs (point j, point j + 8) of real and of imaginary parts.  The
// span-8 stage combines the two halves of each pair (scalar); in the span-4, 2,
// 1 stages the butterflies k and k + 8 share their twiddle, so one packed
// add / subtract / complex multiply serves both.  Twiddles as in fft_dif:
// omega^(2^(3-b)) times a root of unity of order 16; in the last chunk omega = 1
// and the trivial factors (1, i) cost no multiplication.
__device__ __forceinline__ float2 f2(float a) { return make_float2(a, a); }
__device__ __forceinline__ float2 sub2(float2 a, float2 b) { return __ffma2_rn(b, make_float2(-1.f, -1.f), a); }
__device__ __forceinline__ float sin_pi8(int m) { return (float)cos_pi8(m <= 4 ? 4 - m : m - 4); }

// the four stages of one group; TRIV: omega = 1 (last chunk, all twiddles constant)
template <bool TRIV>
__device__ __forceinline__ void bfly16_packed(float2 (&PR)[8], float2 (&PI)[8], float omr, float omi) {
    // span 8: point j with point j + 8, twiddle omega * r16^j
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        const float ar = PR[j].x, cr = PR[j].y, ai = PI[j].x, ci = PI[j].y;
        const float dr = ar - cr, di = ai - ci;
        PR[j].x = ar + cr;
        PI[j].x = ai + ci;
        if (TRIV && j == 0) {
            PR[j].y = dr;
            PI[j].y = di;
        } else if (TRIV && j == 4) {  // times i
            PR[j].y = -di;
            PI[j].y = dr;
        } else {
            float wr = omr, wi = omi;
            if (TRIV) {
                wr = (float)cos_pi8(j);
                wi = sin_pi8(j);
            } else if (j != 0) {
                const float c = (float)cos_pi8(j), sg = sin_pi8(j);
                wr = omr * c - omi * sg;
                wi = omr * sg + omi * c;
            }
            PR[j].y = dr * wr - di * wi;
            PI[j].y = dr * wi + di * wr;
        }
    }
#pragma unroll
    for (int bb = 2; bb >= 0; --bb) {
        if (!TRIV) {  // omega^(2^(3-b))
            const float sr = omr * omr - omi * omi, si = 2.f * omr * omi;
            omr = sr;
            omi = si;
        }
        const int hs = 1 << bb;
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            if (k & hs) continue;
            const int k2 = k | hs;
            const int m = (k & (hs - 1)) << (3 - bb);
            const float2 A = PR[k], C = PR[k2], Ai = PI[k], Ci = PI[k2];
            PR[k] = __fadd2_rn(A, C);
            PI[k] = __fadd2_rn(Ai, Ci);
            const float2 D = sub2(A, C), Di = sub2(Ai, Ci);
            if (TRIV && m == 0) {
                PR[k2] = D;
                PI[k2] = Di;
            } else if (TRIV && m == 4) {  // times i
                PR[k2] = __fmul2_rn(Di, f2(-1.f));
                PI[k2] = D;
            } else {
                float wr = omr, wi = omi;
                if (TRIV) {
                    wr = (float)cos_pi8(m);
                    wi = sin_pi8(m);
                } else if (m != 0) {
                    const float c = (float)cos_pi8(m), sg = sin_pi8(m);
                    wr = omr * c - omi * sg;
                    wi = omr * sg + omi * c;
                }
                PR[k2] = __ffma2_rn(Di, f2(-wi), __fmul2_rn(D, f2(wr)));
                PI[k2] = __ffma2_rn(Di, f2(wr), __fmul2_rn(D, f2(wi)));
            }
        }
    }
}

template <int LGL>
__device__ __forceinline__ void fft_dif_packed(float* tile, const float* cs, const float* sn, int lane, int warp) {
    static_assert(LGL % 4 == 0 && LGL >= 4 && LGL <= 8, "4-bit chunks");
    constexpr int L = 1 << LGL;
    constexpr int NG = L >> 4;                                // groups per chunk
    constexpr int NGW = (NG + LAT_WARPS - 1) / LAT_WARPS;     // groups per warp
    if constexpr (LGL == 8) {  // chunk of bits 7..4 (lo = 4): group data back in place
#pragma unroll
        for (int w = 0; w < NGW; ++w) {
            const int g = warp + w * LAT_WARPS;
            if (g >= NG) break;
            const int base = ((g >> 4) << 8) | (g & 15);
            float2 PR[8], PI[8];
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                const int i0 = base | (j << 4), i1 = base | ((j + 8) << 4);
                PR[j] = make_float2(tile[(2 * i0) * 32 + lane], tile[(2 * i1) * 32 + lane]);
                PI[j] = make_float2(tile[(2 * i0 + 1) * 32 + lane], tile[(2 * i1 + 1) * 32 + lane]);
            }
            const int jt = (g & 15) << (LGL - 7);
            bfly16_packed<false>(PR, PI, cs[jt], sn[jt]);
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                const int i0 = base | (j << 4), i1 = base | ((j + 8) << 4);
                tile[(2 * i0) * 32 + lane] = PR[j].x;
                tile[(2 * i1) * 32 + lane] = PR[j].y;
                tile[(2 * i0 + 1) * 32 + lane] = PI[j].x;
                tile[(2 * i1 + 1) * 32 + lane] = PI[j].y;
            }
        }
        __syncthreads();
    }
    // last chunk (bits 3..0, omega = 1): every group of the warp in registers, then the
    // bit-reversed stores (natural order out)
    float2 PR[NGW][8], PI[NGW][8];
#pragma unroll
    for (int w = 0; w < NGW; ++w) {
        const int g = warp + w * LAT_WARPS;
        if (g >= NG) break;
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const int i0 = g * 16 + j, i1 = g * 16 + j + 8;
            PR[w][j] = make_float2(tile[(2 * i0) * 32 + lane], tile[(2 * i1) * 32 + lane]);
            PI[w][j] = make_float2(tile[(2 * i0 + 1) * 32 + lane], tile[(2 * i1 + 1) * 32 + lane]);
        }
        bfly16_packed<true>(PR[w], PI[w], 1.f, 0.f);
    }
    __syncthreads();  // every input of the last chunk is in registers
#pragma unroll
    for (int w = 0; w < NGW; ++w) {
        const int g = warp + w * LAT_WARPS;
        if (g >= NG) break;
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const int r0 = (int)(__brev((unsigned)(g * 16 + j)) >> (32 - LGL));
            const int r1 = (int)(__brev((unsigned)(g * 16 + j + 8)) >> (32 - LGL));
            tile[(2 * r0) * 32 + lane] = PR[w][j].x;
            tile[(2 * r0 + 1) * 32 + lane] = PI[w][j].x;
            tile[(2 * r1) * 32 + lane] = PR[w][j].y;
            tile[(2 * r1 + 1) * 32 + lane] = PI[w][j].y;
        }
    }
    __syncthreads();
}

template <typename T, int LGL>
__device__ void dst_line(T* tile, const T* tab) {
    constexpr int Nl = 2 << LGL;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    constexpr int L = Nl >> 1;
    const T* cs = tab;
    const T* sn = tab + L;
    const T* sh = tab + Nl;
    // pre-processing: y_j = s_j (x_j + x_{n-j}) + (x_j - x_{n-j}) / 2, y_0 = 0
    for (int j = 1 + warp; j <= L; j += LAT_WARPS) {
        const T a = tile[j * 32 + lane];
        const T b = tile[(Nl - j) * 32 + lane];
        const T s = sh[j] * (a + b);
        const T d = T(0.5) * (a - b);
        tile[j * 32 + lane] = s + d;
        if (j != L) tile[(Nl - j) * 32 + lane] = s - d;
    }
    if (warp == 0) tile[lane] = T(0);
    __syncthreads();
    // complex FFT (sign +) of z_k = (y_2k, y_2k+1), k < L, decimation in frequency
    if constexpr (std::is_same<T, float>::value && LGL % 4 == 0 && LGL <= 8 && !kLatScalarFFT)
        fft_dif_packed<LGL>(tile, cs, sn, lane, warp);  // output in natural order
    else
        fft_dif<T, LGL>(tile, cs, sn, lane, warp);  // output in natural order
    // unpack F_k = E_k + w^k O_k for the pair (k, L-k); write X_2k = Im F_k at 2k,
    // Re F_k at 2k+1 (prefix-summed below)
    for (int k = warp; k <= (L >> 1); k += LAT_WARPS) {
        const int kc = (L - k) & (L - 1);
        T* a = tile + 2 * k * 32 + lane;
        T* c = tile + 2 * kc * 32 + lane;
        const T zr = a[0], zi = a[32], yr = c[0], yi = c[32];
        // E_k = (Z_k + conj Z_{L-k}) / 2 ; O_k = (Z_k - conj Z_{L-k}) / (2i)
        const T er = T(0.5) * (zr + yr), ei = T(0.5) * (zi - yi);
        const T orr = T(0.5) * (zi + yi), oi = T(-0.5) * (zr - yr);
        const T wr = cs[k], wi = sn[k];
        const T fr = er + wr * orr - wi * oi, fi = ei + wr * oi + wi * orr;
        if (kc != k) {
            // F_{L-k}: E_{L-k} = conj E_k, O_{L-k} = conj O_k, w^{L-k} = -conj w^k
            const T gr = er - wr * orr + wi * oi;
            const T gi = -ei + wr * oi + wi * orr;
            c[0] = gi;
            c[32] = gr;
        }
        a[0] = fi;
        a[32] = fr;
    }
    __syncthreads();
    // odd outputs: X_1 = R_0 / 2, X_{2k+1} = X_{2k-1} + R_k  (chunked scan over k)
    __shared__ T part[LAT_WARPS][32];
    const int chunk = (L + LAT_WARPS - 1) / LAT_WARPS;
    const int k0 = warp * chunk, k1 = min(L, k0 + chunk);
    T run = T(0);
    for (int k = k0; k < k1; ++k) run += (k == 0 ? T(0.5) : T(1)) * tile[(2 * k + 1) * 32 + lane];
    part[warp][lane] = run;
    __syncthreads();
    T off = T(0);
    for (int w = 0; w < warp; ++w) off += part[w][lane];
    for (int k = k0; k < k1; ++k) {
        off += (k == 0 ? T(0.5) : T(1)) * tile[(2 * k + 1) * 32 + lane];
        tile[(2 * k + 1) * 32 + lane] = off;
    }
    __syncthreads();
    if (warp == 0) tile[lane] = T(0);
    __syncthreads();
}

template <typename T>
__device__ void load_tab(T* stab, const T* tab, int Nl) {
    for (int i = threadIdx.x; i < Nl + Nl / 2 + 1; i += blockDim.x) stab[i] = tab[i];
}

// row of the lattice point (line, p): pass along x (dir 0) or y (dir 1)
__device__ __forceinline__ size_t lat_row(int dir, int line, int p, int Nl) {
    return dir == 0 ? (size_t)line * (Nl + 1) + p : (size_t)p * (Nl + 1) + line;
}

// LAT_UNROLL points per warp are loaded before any is stored, so that many
// global loads are in flight per warp instead of one
constexpr int LAT_UNROLL = 8;

// the whole tile of a line in flight at once: 16-byte asynchronous copies
// (the row stride is a multiple of 4 values, so a piece never straddles it)
template <typename T>
__device__ void load_line_async(T* tile, const T* __restrict__ in, int dir, int line, int chunk, LatGeom g) {
    constexpr int EPP = 16 / sizeof(T);  // values per piece
    constexpr int PPP = 32 / EPP;        // pieces per point
    const int npieces = (g.Nl - 1) * PPP;
    for (int i = threadIdx.x; i < npieces; i += blockDim.x) {
        const int p = 1 + i / PPP, q = i - (i / PPP) * PPP;
        const int m0 = chunk * 32 + q * EPP;
        T* dst = tile + p * 32 + q * EPP;
        if (m0 < g.ld) {
            const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
            asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(d),
                         "l"(in + lat_row(dir, line, p, g.Nl) * g.ld + m0)
                         : "memory");
        } else {
#pragma unroll
            for (int e = 0; e < EPP; ++e) dst[e] = T(0);
        }
    }
    asm volatile("cp.async.commit_group;" ::: "memory");
    asm volatile("cp.async.wait_group 0;" ::: "memory");
}

template <typename T>
__device__ void load_line(T* tile, const T* __restrict__ in, int dir, int line, int chunk, LatGeom g) {
    if (g.async) {
        load_line_async(tile, in, dir, line, chunk, g);
        return;
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int mode = chunk * 32 + lane;
    for (int p0 = 1 + warp; p0 < g.Nl; p0 += LAT_WARPS * LAT_UNROLL) {
        T v[LAT_UNROLL];
#pragma unroll
        for (int u = 0; u < LAT_UNROLL; ++u) {
            const int p = p0 + u * LAT_WARPS;
            v[u] = (p < g.Nl && mode < g.ld) ? in[lat_row(dir, line, p, g.Nl) * g.ld + mode] : T(0);
        }
#pragma unroll
        for (int u = 0; u < LAT_UNROLL; ++u) {
            const int p = p0 + u * LAT_WARPS;
            if (p < g.Nl) tile[p * 32 + lane] = v[u];
        }
    }
}

// pass X (dir 0) / pass X^-1 (dir 0, store variants)
template <typename T, int LGL>
__global__ void __launch_bounds__(LAT_THREADS)
k_lat_pass_x(const T* __restrict__ in, T* __restrict__ out, const T* __restrict__ tab, LatGeom g, int mode,
             const KrylovScalars* __restrict__ scal) {
    if (scal && scal->done) return;
    extern __shared__ unsigned char smem_raw[];
    T* tile = reinterpret_cast<T*>(smem_raw);
    T* stab = tile + (size_t)g.Nl * 32;
    const int line = 1 + blockIdx.x / g.nchunk, chunk = blockIdx.x % g.nchunk;
    load_tab(stab, tab, g.Nl);
    load_line(tile, in, 0, line, chunk, g);
    __syncthreads();
    dst_line<T, LGL>(tile, stab);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int m = chunk * 32 + lane;
    if (m >= g.ld) return;
    T beta = T(0);
    if (mode == 1 && scal && !scal->first) beta = (T)scal->beta;
    for (int p0 = 1 + warp; p0 < g.Nl; p0 += LAT_WARPS * LAT_UNROLL) {
        T old[LAT_UNROLL];
        if (mode == 1) {
#pragma unroll
            for (int u = 0; u < LAT_UNROLL; ++u) {
                const int p = p0 + u * LAT_WARPS;
                old[u] = (p < g.Nl) ? out[lat_row(0, line, p, g.Nl) * g.ld + m] : T(0);
            }
        }
#pragma unroll
        for (int u = 0; u < LAT_UNROLL; ++u) {
            const int p = p0 + u * LAT_WARPS;
            if (p < g.Nl) {
                const size_t idx = lat_row(0, line, p, g.Nl) * g.ld + m;
                const T z = tile[p * 32 + lane];
                out[idx] = (mode == 1) ? z + beta * old[u] : z;
            }
        }
    }
}

template <typename T, int LGL>
__global__ void __launch_bounds__(LAT_THREADS)
k_lat_pass_y(T* __restrict__ buf, const T* __restrict__ tab, const T* __restrict__ scale, LatGeom g,
             double* __restrict__ rz, const KrylovScalars* __restrict__ scal) {
    if (scal && scal->done) return;
    extern __shared__ unsigned char smem_raw[];
    T* tile = reinterpret_cast<T*>(smem_raw);
    T* stab = tile + (size_t)g.Nl * 32;
    __shared__ double red[LAT_WARPS];
    const int line = 1 + blockIdx.x / g.nchunk, chunk = blockIdx.x % g.nchunk;
    load_tab(stab, tab, g.Nl);
    load_line(tile, buf, 1, line, chunk, g);
    __syncthreads();
    dst_line<T, LGL>(tile, stab);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int N = g.Nl - 1;
    // r'z partial per thread in the working precision (the FP64 pipe is narrow on
    // this GPU), converted to FP64 once per thread below
    T acc_t = T(0);
    for (int p0 = 1 + warp; p0 < g.Nl; p0 += LAT_WARPS * LAT_UNROLL) {
        T sc[LAT_UNROLL];
#pragma unroll
        for (int u = 0; u < LAT_UNROLL; ++u) {
            const int p = p0 + u * LAT_WARPS;
            sc[u] = (p < g.Nl) ? scale[(size_t)(line - 1) * N + (p - 1)] : T(0);
        }
#pragma unroll
        for (int u = 0; u < LAT_UNROLL; ++u) {
            const int p = p0 + u * LAT_WARPS;
            if (p < g.Nl) {
                const T v = tile[p * 32 + lane];
                const T vs = v * sc[u];
                acc_t = fma(v, vs, acc_t);
                tile[p * 32 + lane] = vs;
            }
        }
    }
    double acc = (double)acc_t;
    __syncthreads();
    dst_line<T, LGL>(tile, stab);
    const int m = chunk * 32 + lane;
    if (m < g.ld) {
        for (int p = 1 + warp; p < g.Nl; p += LAT_WARPS)
            buf[lat_row(1, line, p, g.Nl) * g.ld + m] = tile[p * 32 + lane];
    }
    if (rz) {
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
        if (lane == 0) red[warp] = acc;
        __syncthreads();
        if (threadIdx.x == 0) {
            double s = 0.0;
            for (int w = 0; w < LAT_WARPS; ++w) s += red[w];
            rz[blockIdx.x] = s;
        }
    }
}

// Pass Y with the exact mean preconditioner: after pass X the columns kx and
// Nl - kx of the lattice carry the x-frequencies that K_0 couples (the sine
// transform of a stencil that repeats with period 2 links k and Nl - k), so a
// block owns the column pair (i, Nl - i) and 16 modes: lanes 0-15 column i,
// lanes 16-31 column Nl - i (zero when i = Nl/2), each lane one mode.  After
// DST_y the four values of (i | Nl-i) x (ky | Nl-ky) get their 4x4 block of
// (2/Nl)^2 (S K_0 S)^-1, then DST_y again; r'z by Parseval.
template <typename T>
__device__ void load_pair(T* tile, const T* __restrict__ in, int i, int chunk, LatGeom g) {
    const bool self = (2 * i == g.Nl);
    if (g.async) {
        constexpr int EPP = 16 / sizeof(T);
        constexpr int PPH = 16 / EPP;  // pieces per half row of the tile
        const int npieces = (g.Nl - 1) * 2 * PPH;
        for (int t = threadIdx.x; t < npieces; t += blockDim.x) {
            const int p = 1 + t / (2 * PPH), q = t % (2 * PPH), h = q / PPH, qq = q % PPH;
            const int m0 = chunk * 16 + qq * EPP;
            T* dst = tile + p * 32 + h * 16 + qq * EPP;
            if (m0 < g.ld && !(h && self)) {
                const int col = h ? g.Nl - i : i;
                const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
                asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(d),
                             "l"(in + lat_row(1, col, p, g.Nl) * g.ld + m0)
                             : "memory");
            } else {
#pragma unroll
                for (int e = 0; e < EPP; ++e) dst[e] = T(0);
            }
        }
        asm volatile("cp.async.commit_group;" ::: "memory");
        asm volatile("cp.async.wait_group 0;" ::: "memory");
    } else {
        const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, h = lane >> 4;
        const int m = chunk * 16 + (lane & 15), col = h ? g.Nl - i : i;
        const bool ok = m < g.ld && !(h && self);
        for (int p = 1 + warp; p < g.Nl; p += LAT_WARPS)
            tile[p * 32 + lane] = ok ? in[lat_row(1, col, p, g.Nl) * g.ld + m] : T(0);
    }
}

template <typename T, int LGL>
__global__ void __launch_bounds__(LAT_THREADS)
k_lat_pass_yb(T* __restrict__ buf, const T* __restrict__ tab, const T* __restrict__ blk, LatGeom g,
              double* __restrict__ rz, const KrylovScalars* __restrict__ scal) {
    if (scal && scal->done) return;
    extern __shared__ unsigned char smem_raw[];
    T* tile = reinterpret_cast<T*>(smem_raw);
    T* stab = tile + (size_t)g.Nl * 32;
    __shared__ double red[LAT_WARPS];
    const int nc16 = (g.ld + 15) / 16;
    const int i = 1 + blockIdx.x / nc16, chunk = blockIdx.x % nc16;
    const int H = g.Nl / 2;
    load_tab(stab, tab, g.Nl);
    load_pair(tile, buf, i, chunk, g);
    __syncthreads();
    dst_line<T, LGL>(tile, stab);
    T acc_t = T(0);
    for (int item = threadIdx.x; item < H * 16; item += LAT_THREADS) {
        const int ky = 1 + item / 16, m = item % 16;
        const T* q = blk + ((size_t)(i - 1) * H + (ky - 1)) * 10;
        T* pa = tile + ky * 32 + m;
        T* pc = tile + (g.Nl - ky) * 32 + m;
        const T a = pa[0], b = pa[16];
        if (ky != H) {
            const T c = pc[0], d = pc[16];
            const T oa = q[0] * a + q[1] * b + q[2] * c + q[3] * d;
            const T ob = q[1] * a + q[4] * b + q[5] * c + q[6] * d;
            const T oc = q[2] * a + q[5] * b + q[7] * c + q[8] * d;
            const T od = q[3] * a + q[6] * b + q[8] * c + q[9] * d;
            pa[0] = oa;
            pa[16] = ob;
            pc[0] = oc;
            pc[16] = od;
            acc_t = fma(a, oa, fma(b, ob, fma(c, oc, fma(d, od, acc_t))));
        } else {  // ky = Nl - ky: the pair in y collapses
            const T oa = q[0] * a + q[1] * b;
            const T ob = q[1] * a + q[4] * b;
            pa[0] = oa;
            pa[16] = ob;
            acc_t = fma(a, oa, fma(b, ob, acc_t));
        }
    }
    double acc = (double)acc_t;
    __syncthreads();
    dst_line<T, LGL>(tile, stab);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, h = lane >> 4;
    const int m = chunk * 16 + (lane & 15), col = h ? g.Nl - i : i;
    if (m < g.ld && !(h && 2 * i == g.Nl)) {
        for (int p = 1 + warp; p < g.Nl; p += LAT_WARPS) buf[lat_row(1, col, p, g.Nl) * g.ld + m] = tile[p * 32 + lane];
    }
    if (rz) {
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
        if (lane == 0) red[warp] = acc;
        __syncthreads();
        if (threadIdx.x == 0) {
            double s = 0.0;
            for (int w = 0; w < LAT_WARPS; ++w) s += red[w];
            rz[blockIdx.x] = s;
        }
    }
}

LatGeom geom(const sgfem_context* ctx) {
    LatGeom g;
    g.Nl = ctx->Nl;
    g.lg = ctx->lat_log2;
    g.ld = (int)ctx->ld;
    g.nchunk = (int)((ctx->ld + 31) / 32);
    g.async = 0;
    return g;
}

size_t lat_smem(const sgfem_context* ctx, size_t es) {
    return ((size_t)ctx->Nl * 32 + ctx->Nl + ctx->Nl / 2 + 1) * es;
}

// the kernel tables of the including unit
// instantiations for L = Nl/2 = 2^LGL complex points, Nl = 4 .. 512
template <typename T>
sglat::PassXFn<T> local_pass_x_fn(int LGL) {
    switch (LGL) {
        case 1: return k_lat_pass_x<T, 1>;
        case 2: return k_lat_pass_x<T, 2>;
        case 3: return k_lat_pass_x<T, 3>;
        case 4: return k_lat_pass_x<T, 4>;
        case 5: return k_lat_pass_x<T, 5>;
        case 6: return k_lat_pass_x<T, 6>;
        case 7: return k_lat_pass_x<T, 7>;
        case 8: return k_lat_pass_x<T, 8>;
    }
    return nullptr;
}
template <typename T>
sglat::PassYFn<T> local_pass_yb_fn(int LGL) {
    switch (LGL) {
        case 1: return k_lat_pass_yb<T, 1>;
        case 2: return k_lat_pass_yb<T, 2>;
        case 3: return k_lat_pass_yb<T, 3>;
        case 4: return k_lat_pass_yb<T, 4>;
        case 5: return k_lat_pass_yb<T, 5>;
        case 6: return k_lat_pass_yb<T, 6>;
        case 7: return k_lat_pass_yb<T, 7>;
        case 8: return k_lat_pass_yb<T, 8>;
    }
    return nullptr;
}
template <typename T>
sglat::PassYFn<T> local_pass_y_fn(int LGL) {
    switch (LGL) {
        case 1: return k_lat_pass_y<T, 1>;
        case 2: return k_lat_pass_y<T, 2>;
        case 3: return k_lat_pass_y<T, 3>;
        case 4: return k_lat_pass_y<T, 4>;
        case 5: return k_lat_pass_y<T, 5>;
        case 6: return k_lat_pass_y<T, 6>;
        case 7: return k_lat_pass_y<T, 7>;
        case 8: return k_lat_pass_y<T, 8>;
    }
    return nullptr;
}

}  // namespace
