// The two slice-loop passes and the small set-up kernels of the multislice path.
//
// Wave layout: [image][ix][iy], iy contiguous (Kirkland's x-major cfpix,
// multislice/cfpix.hpp:99-125).  One slice of mulslice.cpp:706-739
//     psi *= t;  fft2;  propagate (slicelib.cpp:744-790);  ifft2
// becomes, with the 2D transforms split into their y (row) and x (column) halves,
//     row pass    : ifft_y (finishing the previous slice) -> * t -> fft_y
//     column pass : fft_x -> * py * px, band limit -> ifft_x
// so each slice reads and writes the wave exactly twice (32 * nx * ny bytes per
// probe-slice), and every pointwise step of the reference runs in registers
// between two line transforms.  Kirkland's 1/(nx ny) ifft scale rides in py.
#include <cuda_runtime.h>
#include <atomic>
#include <type_traits>
#include <math.h>
#include <stdint.h>

#include <vector>

#include "msl_fft.cuh"
#include "msl_internal.h"
#include "msl_tma.cuh"

namespace msl {

constexpr int kMaxDet = 8;


template <int N> struct RowCfg {
    using P = Plan<N>;
    static constexpr int LPB = (256 / P::T) > 0 ? 256 / P::T : 1;
    static constexpr int THREADS = P::T * LPB;
    static constexpr size_t SMEM =
        sizeof(float2) * (plan_tw_size<P>() + (size_t)LPB * row_line_slots<P>());
};
template <int N> struct ColCfg {
    using P = Plan<N>;
    static constexpr int C = P::col_c;
    static constexpr int THREADS = P::T * C;
    static constexpr int NWARP = THREADS / 32;
    static constexpr size_t SMEM = sizeof(float2) * (plan_tw_size<P>() + (size_t)N * C) +
                                   sizeof(double) * NWARP * kMaxDet;
};

// ---------------------------------------------------------------- row pass
template <int N>
__global__ void __launch_bounds__(RowCfg<N>::THREADS) row_pass_kernel(RowArgs a) {
    using P = Plan<N>;
    constexpr int T = P::T, E = P::E, LPB = RowCfg<N>::LPB, TW = plan_tw_size<P>();
    extern __shared__ float2 sm[];
    float2 *tw = sm;
    float2 *lines = sm + TW;
    const int tid = threadIdx.x + T * threadIdx.y;
    for (int i = tid; i < TW; i += RowCfg<N>::THREADS) tw[i] = a.tw[i];
    const int t = threadIdx.x;
    RowAddr<P> ad{lines + threadIdx.y * row_line_slots<P>()};
    const int ngroups = (a.nlines + LPB - 1) / LPB;
    for (int g = blockIdx.x; g < ngroups; g += gridDim.x) {
        const int line = g * LPB + threadIdx.y;
        const bool valid = line < a.nlines;
        const size_t base = (size_t)line * N;
        float2 v[E];
        if (valid && (a.flags & ROW_LOAD)) {
#pragma unroll
            for (int e = 0; e < E; ++e) v[e] = a.in[base + t + T * e];
        } else if (valid && (a.flags & ROW_GENT)) {
            // t = exp(i sigma V): phase in FP64, reduced to [-pi, pi] before the
            // single-precision sincos (mulslice.cpp:414-421 forms it in float).
#pragma unroll
            for (int e = 0; e < E; ++e) {
                const double ph = a.phase_scale * (double)a.vpot[base + t + T * e];
                const double k = rint(ph * 0.15915494309189533577);
                const double r = fma(-k, 6.283185307179586477, ph);
                float s, c;
                sincosf((float)r, &s, &c);
                v[e] = make_float2(c, s);
            }
        } else {
#pragma unroll
            for (int e = 0; e < E; ++e) v[e] = make_float2(valid ? 1.f : 0.f, 0.f);
        }
        if (a.flags & ROW_INV) fft_line<P, -1>(v, t, ad, tw);
        if (valid && (a.flags & ROW_TRANS)) {
            const float2 *tr = (a.trans_b ? a.trans_b[line / a.nx] : a.trans) + (size_t)(line % a.nx) * N;
#pragma unroll
            for (int e = 0; e < E; ++e) v[e] = c_mul(v[e], tr[t + T * e]);
        }
        if (a.flags & ROW_FWD) fft_line<P, +1>(v, t, ad, tw);
        if (valid) {
            if (a.scale != 1.0f) {
#pragma unroll
                for (int e = 0; e < E; ++e) v[e] = c_scale(v[e], a.scale);
            }
            if (a.flags & ROW_ACCUM) {
#pragma unroll
                for (int e = 0; e < E; ++e)
                    a.accum[base + t + T * e] +=
                        a.accum_w * ((double)v[e].x * v[e].x + (double)v[e].y * v[e].y);
            }
            if (!(a.flags & ROW_NOSTORE)) {
#pragma unroll
                for (int e = 0; e < E; ++e) a.out[base + t + T * e] = v[e];
            }
        }
    }
}


// --------------------------------------------------- column-pass pointwise
// Reciprocal-space probe of MSProject.cs:458-514: A(k) exp(-i chi) / (nx ny)
// times the two separable position phases.
template <class P>
__device__ __forceinline__ void col_probe(float2 (&v)[P::E], const ColArgs &a, int b, int iy, int t) {
    const float2 eyv = a.ey[(size_t)b * a.ny + iy];
    const float2 *exb = a.ex + (size_t)b * P::N;
#pragma unroll
    for (int e = 0; e < P::E; ++e) {
        const int ix = t + P::T * e;
        v[e] = c_mul(c_mul(a.apchi[(size_t)ix * a.ny + iy], exb[ix]), eyv);
    }
}

// propagate() of slicelib.cpp:744-790: py then px inside the band limit, 0 outside.
template <class P>
__device__ __forceinline__ void col_propagate(float2 (&v)[P::E], const ColArgs &a, int b, int iy, int t) {
    const float2 *px = a.px, *py = a.py;
    const float *kx2 = a.kx2, *ky2t = a.ky2;
    float k2max = a.k2max;
    if (a.prop_b) {  // uneven batches: every image has its own tables
        px = a.prop_b[b];
        py = px + P::N;
        kx2 = a.k2_b[b];
        ky2t = kx2 + P::N;
        k2max = a.k2max_b[b];
    }
    const float ky2 = ky2t[iy];
    const float2 pyv = py[iy];
#pragma unroll
    for (int e = 0; e < P::E; ++e) {
        const int ix = t + P::T * e;
        const float k2 = __fadd_rn(kx2[ix], ky2);
        if (k2 < k2max) v[e] = c_mul(c_mul(v[e], pyv), px[ix]);
        else v[e] = make_float2(0.f, 0.f);
    }
}

// Objective-lens transfer of mulslice.cpp:613-633 from a precomputed table.
template <class P>
__device__ __forceinline__ void col_ctf(float2 (&v)[P::E], const ColArgs &a, int iy, int t) {
#pragma unroll
    for (int e = 0; e < P::E; ++e) v[e] = c_mul(v[e], a.ctf[(size_t)(t + P::T * e) * a.ny + iy]);
}

// Annular detector partial sums of one tile (MSProject.cs:806-829): float per
// thread over its E pixels, then double across the CTA in a fixed order.
template <class P, int NWARP>
__device__ __forceinline__ void col_detect(const float2 (&v)[P::E], const ColArgs &a, int b, int iy,
                                           int t, int ty, int tiles_per_img, double *red) {
    float acc[kMaxDet];
#pragma unroll
    for (int d = 0; d < kMaxDet; ++d) acc[d] = 0.f;
#pragma unroll
    for (int e = 0; e < P::E; ++e) {
        const int ix = t + P::T * e;
        const unsigned bits = a.detmask[(size_t)ix * a.ny + iy];
        const float p = v[e].x * v[e].x + v[e].y * v[e].y;
#pragma unroll
        for (int d = 0; d < kMaxDet; ++d)
            if (bits & (1u << d)) acc[d] += p;
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    __syncthreads();  // red[] of the previous tile has been consumed
#pragma unroll
    for (int d = 0; d < kMaxDet; ++d) {
        if (d < a.ndet) {
            double x = (double)acc[d];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
            if (lane == 0) red[warp * kMaxDet + d] = x;
        }
    }
    __syncthreads();
    if (threadIdx.x < a.ndet) {
        double sum = 0.0;
        for (int w = 0; w < NWARP; ++w) sum += red[w * kMaxDet + threadIdx.x];
        a.partial[((size_t)b * tiles_per_img + ty) * a.ndet + threadIdx.x] = sum;
    }
}

// ------------------------------------------------------------- column pass
template <int N>
__global__ void __launch_bounds__(ColCfg<N>::THREADS) col_pass_kernel(ColArgs a) {
    using P = Plan<N>;
    constexpr int T = P::T, E = P::E, C = P::col_c, TW = plan_tw_size<P>();
    constexpr int NWARP = ColCfg<N>::NWARP;
    extern __shared__ float2 sm[];
    float2 *tw = sm;
    float2 *buf = sm + TW;
    double *red = reinterpret_cast<double *>(buf + (size_t)N * C);
    for (int i = threadIdx.x; i < TW; i += ColCfg<N>::THREADS) tw[i] = a.tw[i];
    const int c = threadIdx.x % C, t = threadIdx.x / C;
    ColAddr<P> ad{buf, c};
    const int tiles_per_img = a.ny / C;
    const int ntiles = a.batch * tiles_per_img;
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int b = tile / tiles_per_img, ty = tile % tiles_per_img;
        const int iy = ty * C + c;
        const size_t base = (size_t)b * N * a.ny + iy;
        float2 v[E];
        if (a.flags & COL_PROBE) {
            col_probe<P>(v, a, b, iy, t);
        } else {
#pragma unroll
            for (int e = 0; e < E; ++e) v[e] = a.in[base + (size_t)(t + T * e) * a.ny];
        }
        if (a.flags & COL_FWD) fft_line<P, +1>(v, t, ad, tw);
        if (a.flags & COL_PROP) col_propagate<P>(v, a, b, iy, t);
        if (a.flags & COL_CTF) col_ctf<P>(v, a, iy, t);
        if (a.flags & COL_DETECT) col_detect<P, NWARP>(v, a, b, iy, t, ty, tiles_per_img, red);
        if (a.flags & COL_INV) fft_line<P, -1>(v, t, ad, tw);
        if (a.flags & COL_STORE) {
#pragma unroll
            for (int e = 0; e < E; ++e) a.out[base + (size_t)(t + T * e) * a.ny] = v[e];
        }
    }
}


// ------------------------------------------------- TMA-fed column pass
// Persistent kernel, as many CTAs per SM as the plan's MINB and its shared
// memory allow.  Column tiles of C columns x N rows (C * 8 bytes wide) arrive by
// cp.async.bulk.tensor into a ring of NBUF shared-memory buffers (three: while
// tile k is transformed in buffer k % 3, tile k+1 is already resident and tile
// k+2 is in flight; two: tile k+1 loads while tile k is transformed).  The same
// buffer then serves as the transform's exchange space and as the source of
// the TMA store of the result, so a tile never touches registers-to-global
// stores.  Every mbarrier wait is bounded; on a timeout the CTA raises *err,
// waits (bounded) for its loads still in flight and leaves.
constexpr uint32_t kWaitLimit = 1u << 22;

template <class A> __device__ __forceinline__ A make_col_addr(float2 *bs, int c) {
    if constexpr (is_col_lin<A>::value) return A{smem_u32(bs) + 8u * (uint32_t)c};
    else return A{bs, c};
}

template <class PL> struct ColTmaCfg {
    using P = PL;
    static constexpr int N = P::N;
    static constexpr int C = P::col_c, T = P::T, THREADS = T * C, NWARP = THREADS / 32;
    static constexpr int NBUF = P::NBUF;
    static_assert(NBUF >= 2 && NBUF <= 4, "tile ring of two to four buffers");
    // rows per TMA box: the largest divisor of N not above 256 (the box limit)
    static constexpr int BOXR = N <= 256 ? N : (N % 256 == 0 ? 256 : N / 2), NBOX = N / BOXR;
    static_assert(BOXR <= 256 && BOXR * NBOX == N, "TMA boxes must tile the column");
    static constexpr size_t TILE_BYTES = sizeof(float2) * (size_t)N * C;
    static constexpr size_t OFF_TW = NBUF * TILE_BYTES;
    static constexpr size_t OFF_RED = OFF_TW + ((sizeof(float2) * plan_tw_size<P>() + 15) / 16) * 16;
    static constexpr size_t OFF_BAR = OFF_RED + sizeof(double) * NWARP * kMaxDet;
    static constexpr size_t SMEM = OFF_BAR + sizeof(uint64_t) * NBUF + 1024;  // + base alignment
};

template <class PL, int MINB>
__global__ void __launch_bounds__(ColTmaCfg<PL>::THREADS, MINB)
    col_tma_kernel(const __grid_constant__ CUtensorMap map, ColArgs a) {
    using Cfg = ColTmaCfg<PL>;
    using P = PL;
    constexpr int N = P::N;
    constexpr int C = Cfg::C, T = P::T, E = P::E, TW = plan_tw_size<P>(), NBUF = Cfg::NBUF;
    extern __shared__ unsigned char smraw[];
    unsigned char *base = smraw + ((1024u - (smem_u32(smraw) & 1023u)) & 1023u);
    float2 *buf0 = reinterpret_cast<float2 *>(base);
    float2 *tw = reinterpret_cast<float2 *>(base + Cfg::OFF_TW);
    double *red = reinterpret_cast<double *>(base + Cfg::OFF_RED);
    uint64_t *bar = reinterpret_cast<uint64_t *>(base + Cfg::OFF_BAR);
    const int tid = threadIdx.x, c = tid % C, t = tid / C;
    const bool load = (a.flags & COL_LOAD) != 0, store = (a.flags & COL_STORE) != 0;
    const int tpi = a.ny / C, ntiles = a.batch * tpi;
    const int nmine = (ntiles - (int)blockIdx.x + (int)gridDim.x - 1) / (int)gridDim.x;
    if constexpr (P::OWN_TW) {  // stage s >= 1: [r][k] = exp(2 pi i r k / (NS R)), NS = span before s
#pragma unroll
        for (int st = 1; st < P::NSTAGE; ++st) {
            const int R = P::radix(st), NS = plan_span<P>(st), off = plan_tw_offset<P>(st);
            for (int i = tid; i < R * NS; i += Cfg::THREADS) {
                float sn, cn;
                sincospif((float)(2 * (i / NS) * (i % NS)) / (float)(NS * R), &sn, &cn);
                tw[off + i] = make_float2(cn, sn);
            }
        }
    } else {
        for (int i = tid; i < TW; i += Cfg::THREADS) tw[i] = a.tw[i];
    }
    if (tid == 0) {
        for (int s = 0; s < NBUF; ++s) mbar_init(&bar[s], 1);
        mbar_fence_init();
    }
    __syncthreads();
    int issued = 0;  // loads issued (thread 0's count)
    auto issue_load = [&](int k) {
        const int tile = blockIdx.x + k * gridDim.x, b = tile / tpi, ty = tile % tpi, s = k % NBUF;
        float2 *dst = buf0 + (size_t)s * N * C;
        fence_proxy_async();
        mbar_arrive_expect_tx(&bar[s], (uint32_t)Cfg::TILE_BYTES);
#pragma unroll
        for (int q = 0; q < Cfg::NBOX; ++q)
            tma_load_2d(dst + (size_t)q * Cfg::BOXR * C, &map, ty * C, b * N + q * Cfg::BOXR, &bar[s]);
        issued = k + 1;
    };
    if (load && tid == 0)
        for (int k = 0; k < NBUF - 1 && k < nmine; ++k) issue_load(k);
    int k = 0;
    bool ok = true;
    for (; k < nmine; ++k) {
        const int tile = blockIdx.x + k * gridDim.x, b = tile / tpi, ty = tile % tpi;
        const int iy = ty * C + c, s = k % NBUF;
        float2 *bs = buf0 + (size_t)s * N * C;
        using Addr = typename std::conditional<(N & (N - 1)) == 0, ColXorLin<P>, ColAddr<P>>::type;
        Addr ad = make_col_addr<Addr>(bs, c);
        float2 v[E];
        if (!load && store && tid == 0) tma_wait_read<NBUF - 1>();  // store of tile k-NBUF left bs
        if (load) {
            const bool got = mbar_wait_bounded(&bar[s], (uint32_t)((k / NBUF) & 1), kWaitLimit);
            if (__syncthreads_or(!got)) {
                ok = false;
                break;
            }
            if constexpr (NBUF == 2) {
                // two buffers: tile k+1 goes into the buffer of tile k-1 once every
                // thread is past it (the barrier above) and its store has read it,
                // so it loads while tile k is transformed
                if (tid == 0 && k + 1 < nmine) {
                    if (store) tma_wait_read<0>();
                    issue_load(k + 1);
                }
            }
#pragma unroll
            for (int e = 0; e < E; ++e) v[e] = bs[(t + T * e) * C + c];
        } else if (a.flags & COL_PROBE) {
            col_probe<P>(v, a, b, iy, t);
        } else {
#pragma unroll
            for (int e = 0; e < E; ++e) v[e] = make_float2(0.f, 0.f);
        }
        if (a.flags & COL_FWD) fft_line<P, +1>(v, t, ad, tw);
        if (a.flags & COL_PROP) col_propagate<P>(v, a, b, iy, t);
        if (a.flags & COL_CTF) col_ctf<P>(v, a, iy, t);
        if (a.flags & COL_DETECT) col_detect<P, Cfg::NWARP>(v, a, b, iy, t, ty, tpi, red);
        if (a.flags & COL_INV) fft_line<P, -1>(v, t, ad, tw);
        if (store) {
            __syncthreads();  // every thread is done reading bs
#pragma unroll
            for (int e = 0; e < E; ++e) bs[(t + T * e) * C + c] = v[e];
            fence_proxy_async();
            __syncthreads();
            if (tid == 0) {
#pragma unroll
                for (int q = 0; q < Cfg::NBOX; ++q)
                    tma_store_2d(&map, ty * C, b * N + q * Cfg::BOXR, bs + (size_t)q * Cfg::BOXR * C);
                tma_commit();
            }
        }
        if constexpr (NBUF >= 3) {
            if (load && tid == 0 && k + NBUF - 1 < nmine) {
                if (store) tma_wait_read<1>();  // the store of tile k-1 has left its buffer
                issue_load(k + NBUF - 1);       // into the buffer of tile k-1
            }
        }
    }
    if (tid == 0) {
        if (store) tma_wait_all();
        if (!ok) {
            if (a.err) atomicExch(a.err, 1);
            // loads still in flight land in this CTA's shared memory: let them finish
            for (int j = k; j < issued; ++j)
                mbar_wait_bounded(&bar[j % NBUF], (uint32_t)((j / NBUF) & 1), kWaitLimit);
        }
    }
}


// ------------------------- column pass, two-stage columns, 256 / 512 / 1024
// The slice loop's column passes at N = 256, 512 and 1024 built like the
// two-stage row pass: each column is one line of T threads x E elements
// (radix 16 x 16 at 256, 16 x 32 at 512, 32 x 32 at 1024), one exchange per
// transform.  Tiles of C columns x N rows (16 KB at 256, else 32 KB) arrive by
// TMA with a swizzle (ColLin64, ColLin32) under which the natural-order reads
// and writes of the tile are conflict-free; the exchange reuses each column's
// own slots in a permuted order, conflict-free too.  At 256 and 512 a warp owns
// two columns (16 lanes each, alternating) and its exchanges need only the
// warp; at 1024 a warp pair owns two columns (16 lanes of each warp per column)
// and syncs on a named barrier of 64 threads.  One CTA per SM runs G groups of
// 4 warps; each group streams its own tiles through a two-slot ring of
// slot-aligned buffers (every exchange address is a per-thread base xor a
// constant).  Group barriers per tile: the arrival vote and the one before the
// TMA store (two more at detector checkpoints).  Detector partial sums are
// written per 4 columns.
struct ColHalfL512 {  // 512: 8 columns, a warp per column pair
    using P = HalfWarpColPlan512;
    using Lin = ColLin64;
    static constexpr int N = 512, C = 8, G = 3, WPG = 4;
    static constexpr bool PAIR = false;
    static constexpr CUtensorMapSwizzle SWZ = CU_TENSOR_MAP_SWIZZLE_64B;
    __device__ static int col(int wg, int lane) { return 2 * wg + (lane & 1); }
    __device__ static int thr(int wg, int lane) { return lane >> 1; }
};
struct ColHalfL256 {  // 256: 8 columns, a warp per column pair, four groups per CTA
    using P = HalfWarpColPlan256;
    using Lin = ColLin64;
    static constexpr int N = 256, C = 8, G = 4, WPG = 4;
    static constexpr bool PAIR = false;
    static constexpr CUtensorMapSwizzle SWZ = CU_TENSOR_MAP_SWIZZLE_64B;
    __device__ static int col(int wg, int lane) { return 2 * wg + (lane & 1); }
    __device__ static int thr(int wg, int lane) { return lane >> 1; }
};
struct ColPairL1024 {  // 1024: 4 columns, a warp pair per column pair
    using P = WarpPairColPlan1024;
    using Lin = ColLin32;
    static constexpr int N = 1024, C = 4, G = 3, WPG = 4;
    static constexpr bool PAIR = true;
    static constexpr CUtensorMapSwizzle SWZ = CU_TENSOR_MAP_SWIZZLE_32B;
    __device__ static int col(int wg, int lane) { return 2 * (wg >> 1) + (lane & 1); }
    __device__ static int thr(int wg, int lane) { return 16 * (wg & 1) + (lane >> 1); }
};

template <class L> struct ColHalfCfg {
    using P = typename L::P;
    static constexpr int N = L::N, C = L::C, G = L::G, GT = 32 * L::WPG, THREADS = GT * G, NBUF = 2, BOXR = 256;
    static constexpr uint32_t SLOT = sizeof(float2) * N * C;  // 16 or 32 KB, also the slot alignment
    static constexpr int TW = P::radix(1) * P::radix(0);      // stage 1 table [r][k]
    static constexpr size_t OFF_RED = sizeof(float2) * TW;
    static constexpr size_t OFF_BAR = OFF_RED + sizeof(double) * G * L::WPG * kMaxDet;
    static constexpr size_t HEADER = OFF_BAR + sizeof(uint64_t) * G * NBUF;
    // the header, then 2 G slots from the next slot boundary
    static constexpr size_t SMEM = HEADER + SLOT - 1 + (size_t)NBUF * G * SLOT + 1024 <= 227 * 1024
                                       ? HEADER + SLOT - 1 + (size_t)NBUF * G * SLOT + 1024 : 227 * 1024;
    static_assert((SLOT & (SLOT - 1)) == 0 && N % BOXR == 0 && P::NSTAGE == 2 && C % 4 == 0, "two stages");
    static_assert(1 + G + (L::PAIR ? 2 * G : 0) <= 16, "named barriers: one per group, one per warp pair");
    // natural order: row t + T e of a column at nb + e ROWSTEP, nb the thread's base
    static constexpr uint32_t ROWSTEP = L::Lin::B(P::T);
    static_assert(L::Lin::B(P::T - 1) < ROWSTEP && L::Lin::B(3 * P::T) == 3 * ROWSTEP, "natural-order stride");
    static_assert(HEADER <= SLOT, "the header fits before the first slot");
};

template <class L>
__global__ void __launch_bounds__(ColHalfCfg<L>::THREADS, 1)
    col_half_kernel(const __grid_constant__ CUtensorMap map, ColArgs a) {
    using Cfg = ColHalfCfg<L>;
    using P = typename Cfg::P;
    using Lin = typename L::Lin;
    constexpr int N = Cfg::N, C = Cfg::C, E = P::E, T = P::T, G = Cfg::G, GT = Cfg::GT, NBUF = Cfg::NBUF;
    constexpr int R0 = P::radix(0);
    constexpr uint32_t SLOT = Cfg::SLOT;
    extern __shared__ unsigned char smraw[];
    const uint32_t sbase = smem_u32(smraw);
    const uint32_t slot0 = (sbase + (uint32_t)Cfg::HEADER + SLOT - 1u) & ~(SLOT - 1u);
    if (slot0 + (uint32_t)(NBUF * G) * SLOT > sbase + (uint32_t)Cfg::SMEM) {  // uniform over the CTA
        if (threadIdx.x == 0 && a.err) atomicExch(a.err, 2);                  // layout error, not a timeout
        return;
    }
    float2 *tw = reinterpret_cast<float2 *>(smraw);
    double *redall = reinterpret_cast<double *>(smraw + Cfg::OFF_RED);
    uint64_t *barall = reinterpret_cast<uint64_t *>(smraw + Cfg::OFF_BAR);
    for (int i = threadIdx.x; i < Cfg::TW; i += Cfg::THREADS) {
        float sn, cn;
        sincospif((float)(2 * (i / R0) * (i % R0)) / (float)N, &sn, &cn);  // exp(2 pi i r k / N), [r][k]
        tw[i] = make_float2(cn, sn);
    }
    const float2 *twp = P::GTW ? a.tw + P::GTW_OFF : tw;
    if (threadIdx.x == 0) {
        for (int s = 0; s < G * NBUF; ++s) mbar_init(&barall[s], 1);
        mbar_fence_init();
    }
    __syncthreads();  // the only CTA-wide barrier
    const int g = threadIdx.x / GT, gt = threadIdx.x % GT, wg = gt >> 5, lane = gt & 31;
    // lanes alternate between two columns: each half-warp then touches 8 rows of
    // both, which is what keeps its 64-bit accesses on 16 bank pairs
    const int t = L::thr(wg, lane), c = L::col(wg, lane);
    const uint32_t pairid = 1u + G + 2u * (uint32_t)g + (uint32_t)(wg >> 1);  // the warp pair's barrier (1024)
    auto colsync = [&]() {
        if constexpr (L::PAIR) bar_group(pairid, 64);
        else __syncwarp();
    };
    const uint32_t barid = 1u + (uint32_t)g;
    uint64_t *bar = barall + g * NBUF;
    double *red = redall + g * L::WPG * kMaxDet;
    const uint32_t gslot = slot0 + (uint32_t)(g * NBUF) * SLOT;
    const bool store = (a.flags & COL_STORE) != 0;
    const int tpi = a.ny / C, ntiles = a.batch * tpi;
    const int NG = gridDim.x * G, gid = blockIdx.x * G + g;
    const int nmine = gid < ntiles ? (ntiles - gid + NG - 1) / NG : 0;
    int issued = 0;
    auto issue = [&](int k) {  // group thread 0 only
        const int tile = gid + k * NG, b = tile / tpi, ty = tile % tpi, s = k % NBUF;
        unsigned char *dst = smraw + (gslot + (uint32_t)s * SLOT - sbase);
        fence_proxy_async();
        mbar_arrive_expect_tx(&bar[s], SLOT);
#pragma unroll
        for (int q = 0; q < N / Cfg::BOXR; ++q)
            tma_load_2d(dst + (size_t)q * Cfg::BOXR * C * sizeof(float2), &map, ty * C, b * N + q * Cfg::BOXR,
                        &bar[s]);
        issued = k + 1;
    };
    if (gt == 0 && nmine > 0) issue(0);
    int k = 0;
    bool ok = true;
    for (; k < nmine; ++k) {
        const int tile = gid + k * NG, b = tile / tpi, ty = tile % tpi, s = k % NBUF;
        if (gt == 0 && k + 1 < nmine) {
            if (store) tma_wait_read<0>();  // the store of tile k-1 has read the other slot
            issue(k + 1);
        }
        const bool got = mbar_wait_bounded(&bar[s], (uint32_t)((k / NBUF) & 1), kWaitLimit);
        if (bar_group_or(barid, GT, !got)) {
            ok = false;
            break;
        }
        const uint32_t cb = (gslot + (uint32_t)s * SLOT) ^ (8u * (uint32_t)c);
        const uint32_t nb = cb ^ Lin::B((uint32_t)t);  // row t + T e at nb + ROWSTEP e
        float2 v[E];
#pragma unroll
        for (int e = 0; e < E; ++e) v[e] = lds_f2(nb + Cfg::ROWSTEP * (uint32_t)e);
        fft_stage<P, 0, +1>(v, t, tw);
        fft_exchange_ch<P, 0, Lin>(v, t, cb, colsync);
        fft_stage<P, 1, +1>(v, t, tw);
        const int iy = ty * C + c;
        if (a.flags & COL_PROP) col_propagate<P>(v, a, b, iy, t);
        if (a.flags & COL_CTF) col_ctf<P>(v, a, iy, t);
        if (a.flags & COL_DETECT) {
            float acc[kMaxDet];
#pragma unroll
            for (int d = 0; d < kMaxDet; ++d) acc[d] = 0.f;
#pragma unroll
            for (int e = 0; e < E; ++e) {
                const unsigned bits = a.detmask[(size_t)(t + T * e) * a.ny + iy];
                const float p = v[e].x * v[e].x + v[e].y * v[e].y;
#pragma unroll
                for (int d = 0; d < kMaxDet; ++d)
                    if (bits & (1u << d)) acc[d] += p;
            }
            bar_group(barid, GT);  // red[] of the previous tile has been consumed
#pragma unroll
            for (int d = 0; d < kMaxDet; ++d) {
                if (d < a.ndet) {
                    double x = (double)acc[d];
#pragma unroll
                    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
                    if (lane == 0) red[wg * kMaxDet + d] = x;
                }
            }
            bar_group(barid, GT);
            constexpr int NBLK = C / 4, WPB = L::WPG / NBLK;  // 4-column blocks per tile, warps per block
            if (gt < NBLK * a.ndet) {                   // warps WPB hq .. WPB hq + WPB - 1 hold block hq
                const int hq = gt / a.ndet, d = gt % a.ndet;
                double sum = 0.0;
#pragma unroll
                for (int w = 0; w < WPB; ++w) sum += red[(WPB * hq + w) * kMaxDet + d];
                a.partial[((size_t)b * (a.ny / 4) + NBLK * ty + hq) * a.ndet + d] = sum;
            }
        }
        if (a.flags & COL_INV) {  // absent on a scan's last slice (detection only)
            fft_stage<P, 0, -1>(v, t, tw);
            fft_exchange_ch<P, 0, Lin>(v, t, cb, colsync);
            fft_stage<P, 1, -1>(v, t, tw);
        }
        if (store) {
            colsync();  // every thread of the columns is done reading them
#pragma unroll
            for (int e = 0; e < E; ++e) sts_f2(nb + Cfg::ROWSTEP * (uint32_t)e, v[e]);
            fence_proxy_async();
            bar_group(barid, GT);
            if (gt == 0) {
                const unsigned char *src = smraw + (gslot + (uint32_t)s * SLOT - sbase);
#pragma unroll
                for (int q = 0; q < N / Cfg::BOXR; ++q)
                    tma_store_2d(&map, ty * C, b * N + q * Cfg::BOXR, src + (size_t)q * Cfg::BOXR * C * sizeof(float2));
                tma_commit();
            }
        } else {
            bar_group(barid, GT);  // the slot is free before the load of tile k + 2 lands in it
        }
    }
    if (gt == 0) {
        if (store) tma_wait_all();
        if (!ok) {
            if (a.err) atomicExch(a.err, 1);
            for (int j = k; j < issued; ++j)
                mbar_wait_bounded(&bar[j % NBUF], (uint32_t)((j / NBUF) & 1), kWaitLimit);
        }
    }
}

// ---------------------------------------------------- TMA-fed row pass
// Persistent kernel, MINB CTAs per SM, TH threads = L lines x T threads.  Tiles
// of L consecutive lines (L * N * 8 bytes, contiguous) arrive by TMA into a ring
// of three buffers; the buffer is then the line transforms' exchange space and
// the source of the TMA store.  The tile is viewed as [L][N/BX][BX] so every box
// dimension stays within the 256-element TMA limit while the shared-memory
// image of the tile is plain [line][N].  The transmission row of each line is
// read straight from global memory (it is shared by the whole probe batch and
// sits in L2) at the start of the tile, so its latency overlaps the inverse
// transform.
template <int N, int TH> struct RowTmaCfg {
    using P = Plan<N>;
    static constexpr int T = P::T, L = TH / T, THREADS = T * L;
    static constexpr int NBUF = 3;
    static constexpr int BX = N <= 256 ? N : (N % 256 == 0 ? 256 : N / 2), NBX = N / BX;
    static_assert(BX <= 256 && BX * NBX == N && NBX <= 256 && L <= 256, "TMA box limits");
    static constexpr size_t TILE_BYTES = sizeof(float2) * (size_t)L * N;
    static constexpr size_t OFF_TW = NBUF * TILE_BYTES;
    static constexpr size_t OFF_BAR = OFF_TW + ((sizeof(float2) * plan_tw_size<P>() + 15) / 16) * 16;
    static constexpr size_t SMEM = OFF_BAR + sizeof(uint64_t) * NBUF + 1024;
};

template <int N, int TH, int MINB>
__global__ void __launch_bounds__(RowTmaCfg<N, TH>::THREADS, MINB)
    row_tma_kernel(const __grid_constant__ CUtensorMap map, RowArgs a) {
    using Cfg = RowTmaCfg<N, TH>;
    using P = Plan<N>;
    constexpr int T = P::T, E = P::E, L = Cfg::L, TW = plan_tw_size<P>(), NBUF = Cfg::NBUF;
    extern __shared__ unsigned char smraw[];
    unsigned char *base = smraw + ((1024u - (smem_u32(smraw) & 1023u)) & 1023u);
    float2 *buf0 = reinterpret_cast<float2 *>(base);
    float2 *tw = reinterpret_cast<float2 *>(base + Cfg::OFF_TW);
    uint64_t *bar = reinterpret_cast<uint64_t *>(base + Cfg::OFF_BAR);
    const int tid = threadIdx.x, t = tid % T, l = tid / T;
    const bool load = (a.flags & ROW_LOAD) != 0;
    const int ntiles = a.nlines / L;
    const int nmine = (ntiles - (int)blockIdx.x + (int)gridDim.x - 1) / (int)gridDim.x;
    for (int i = tid; i < TW; i += Cfg::THREADS) tw[i] = a.tw[i];
    if (tid == 0) {
        for (int s = 0; s < NBUF; ++s) mbar_init(&bar[s], 1);
        mbar_fence_init();
    }
    __syncthreads();
    int issued = 0;
    auto issue_load = [&](int k) {
        const int tile = blockIdx.x + k * gridDim.x, s = k % NBUF;
        fence_proxy_async();
        mbar_arrive_expect_tx(&bar[s], (uint32_t)Cfg::TILE_BYTES);
        tma_load_3d(buf0 + (size_t)s * L * N, &map, 0, 0, tile * L, &bar[s]);
        issued = k + 1;
    };
    if (load && tid == 0)
        for (int k = 0; k < NBUF - 1 && k < nmine; ++k) issue_load(k);
    int k = 0;
    bool ok = true;
    for (; k < nmine; ++k) {
        const int tile = blockIdx.x + k * gridDim.x, s = k % NBUF;
        const int line = tile * L + l;
        float2 *bs = buf0 + (size_t)s * L * N;
        float2 *mine = bs + (size_t)l * N;
        RowXorAddr<P> ad{mine};
        float2 tr[E];
        if (a.flags & ROW_TRANS) {
            const float2 *trow = (a.trans_b ? a.trans_b[line / a.nx] : a.trans) + (size_t)(line % a.nx) * N;
#pragma unroll
            for (int e = 0; e < E; ++e) tr[e] = __ldg(trow + t + T * e);
        }
        if (tid == 0) tma_wait_read<NBUF - 1>();  // the store of tile k-3 has left bs
        float2 v[E];
        if (load) {
            const bool got = mbar_wait_bounded(&bar[s], (uint32_t)((k / NBUF) & 1), kWaitLimit);
            if (__syncthreads_or(!got)) {
                ok = false;
                break;
            }
#pragma unroll
            for (int e = 0; e < E; ++e) v[e] = mine[t + T * e];
        } else {
#pragma unroll
            for (int e = 0; e < E; ++e) v[e] = make_float2(1.f, 0.f);
        }
        if (a.flags & ROW_INV) fft_line<P, -1>(v, t, ad, tw);
        if (a.flags & ROW_TRANS) {
#pragma unroll
            for (int e = 0; e < E; ++e) v[e] = c_mul(v[e], tr[e]);
        }
        if (a.flags & ROW_FWD) fft_line<P, +1>(v, t, ad, tw);
        if (a.scale != 1.0f) {
#pragma unroll
            for (int e = 0; e < E; ++e) v[e] = c_scale(v[e], a.scale);
        }
        if (a.flags & ROW_ACCUM) {
            double *acc = a.accum + (size_t)line * N;
#pragma unroll
            for (int e = 0; e < E; ++e)
                acc[t + T * e] += a.accum_w * ((double)v[e].x * v[e].x + (double)v[e].y * v[e].y);
        }
        const bool st = !(a.flags & ROW_NOSTORE);
        __syncthreads();  // every thread is done reading bs
        if (st) {
#pragma unroll
            for (int e = 0; e < E; ++e) mine[t + T * e] = v[e];
            fence_proxy_async();
        }
        __syncthreads();
        if (tid == 0) {
            if (st) {
                tma_store_3d(&map, 0, 0, tile * L, bs);
                tma_commit();
            }
            if (load && k + NBUF - 1 < nmine) {
                tma_wait_read<1>();        // the store of tile k-1 has left its buffer
                issue_load(k + NBUF - 1);  // into buffer (k + 2) % 3
            }
        }
    }
    if (tid == 0) {
        tma_wait_all();
        if (!ok) {
            if (a.err) atomicExch(a.err, 1);
            for (int j = k; j < issued; ++j)
                mbar_wait_bounded(&bar[j % NBUF], (uint32_t)((j / NBUF) & 1), kWaitLimit);
        }
    }
}


// ---------------------- warp-per-line row pass (half-warp lines at 384)
// Persistent kernel in which every warp owns whole lines (one, or two
// half-warp lines when the plan has 16 threads per line): it streams them
// through its own two- or three-slot ring in shared memory with 1D bulk copies
// (cp.async.bulk) and its own mbarriers, and the line transforms exchange
// through that ring with warp-level synchronisation only.  No CTA-wide barrier
// runs after the prologue, so a warp waiting on its exchange or its next line
// never holds up the others.
template <class A> __device__ __forceinline__ A make_row_addr(float2 *buf);
template <> __device__ __forceinline__ RowXorLin<WarpPlan<256>> make_row_addr(float2 *buf) {
    return RowXorLin<WarpPlan<256>>{smem_u32(buf)};
}
template <> __device__ __forceinline__ RowXorLin<WarpPlan<512>> make_row_addr(float2 *buf) {
    return RowXorLin<WarpPlan<512>>{smem_u32(buf)};
}
template <> __device__ __forceinline__ RowXorAddr<WarpPlan<384>> make_row_addr(float2 *buf) {
    return RowXorAddr<WarpPlan<384>>{buf};
}
template <> __device__ __forceinline__ RowXorAddr<WarpPlan<768>> make_row_addr(float2 *buf) {
    return RowXorAddr<WarpPlan<768>>{buf};
}

template <int N> struct RowWarpCfg {
    using P = WarpPlan<N>;
    static constexpr int LPW = 32 / P::T;  // lines per warp: 1, or 2 for half-warp lines
    static constexpr int W = 8, THREADS = 32 * W, NBUF = (N == 512 || N == 768 || LPW > 1) ? 2 : 3;
    static constexpr int MINB = N == 512 ? 3 : P::E <= 8 ? 3 : 2;
    static constexpr size_t LINE = sizeof(float2) * N, UNIT = LPW * LINE;
    // power-of-two sides address their exchanges xor-linearly (RowXorLin), which
    // needs every line buffer aligned to its size
    static constexpr bool XL = (N & (N - 1)) == 0;
    static constexpr uint32_t ALIGN = XL ? (uint32_t)LINE : 128u;
    static constexpr size_t OFF_TW = (size_t)W * NBUF * UNIT;
    static constexpr size_t OFF_BAR = OFF_TW + ((sizeof(float2) * plan_tw_size<P>() + 15) / 16) * 16;
    static constexpr size_t SMEM = OFF_BAR + sizeof(uint64_t) * W * NBUF + ALIGN;
    static_assert(P::T == 32 || P::T == 16, "warp- or half-warp-owned lines");
};

template <int N>
__global__ void __launch_bounds__(RowWarpCfg<N>::THREADS, RowWarpCfg<N>::MINB) row_warp_kernel(RowArgs a) {
    using Cfg = RowWarpCfg<N>;
    using P = WarpPlan<N>;
    constexpr int E = P::E, T = P::T, LPW = Cfg::LPW, NBUF = Cfg::NBUF, W = Cfg::W, TW = plan_tw_size<P>();
    constexpr uint32_t AL = Cfg::ALIGN;
    extern __shared__ unsigned char smraw[];
    unsigned char *base = smraw + ((AL - (smem_u32(smraw) & (AL - 1u))) & (AL - 1u));
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, h = lane / T, t = lane % T;
    float2 *ring = reinterpret_cast<float2 *>(base) + (size_t)warp * NBUF * LPW * N;
    float2 *tw = reinterpret_cast<float2 *>(base + Cfg::OFF_TW);
    uint64_t *bar = reinterpret_cast<uint64_t *>(base + Cfg::OFF_BAR) + warp * NBUF;
    if constexpr (P::OWN_TW) {  // stage s >= 1: [r][k] = exp(2 pi i r k / (NS R)), NS = span before s
#pragma unroll
        for (int st = 1; st < P::NSTAGE; ++st) {
            const int R = P::radix(st), NS = plan_span<P>(st), off = plan_tw_offset<P>(st);
            for (int i = threadIdx.x; i < R * NS; i += Cfg::THREADS) {
                float sn, cn;
                sincospif((float)(2 * (i / NS) * (i % NS)) / (float)(NS * R), &sn, &cn);
                tw[off + i] = make_float2(cn, sn);
            }
        }
    } else {
        for (int i = threadIdx.x; i < TW; i += Cfg::THREADS) tw[i] = a.tw[i];
    }
    if (lane == 0) {
        for (int s = 0; s < NBUF; ++s) mbar_init(&bar[s], 1);
        mbar_fence_init();
    }
    __syncthreads();  // the only CTA barrier: tables and barriers are ready
    const bool load = (a.flags & ROW_LOAD) != 0, store = !(a.flags & ROW_NOSTORE);
    const int nunits = a.nlines / LPW;  // units of LPW consecutive lines, one per warp at a time
    const int G = gridDim.x * W, gw = blockIdx.x * W + warp;
    const int nmine = gw < nunits ? (nunits - gw + G - 1) / G : 0;
    int issued = 0;
    auto issue = [&](int k) {  // lane 0 only
        const int unit = gw + k * G, s = k % NBUF;
        fence_proxy_async();
        mbar_arrive_expect_tx(&bar[s], (uint32_t)Cfg::UNIT);
        bulk_load(ring + (size_t)s * LPW * N, a.in + (size_t)unit * LPW * N, (uint32_t)Cfg::UNIT, &bar[s]);
        issued = k + 1;
    };
    if (load && lane == 0)
        for (int k = 0; k < NBUF - 1 && k < nmine; ++k) issue(k);
    int k = 0;
    bool ok = true;
    for (; k < nmine; ++k) {
        const int unit = gw + k * G, s = k % NBUF, line = LPW * unit + h;
        float2 *slot = ring + (size_t)s * LPW * N;
        float2 *buf = slot + (size_t)h * N;
        using Addr = typename std::conditional<Cfg::XL, RowXorLin<P>, RowXorAddr<P>>::type;
        Addr ad = make_row_addr<Addr>(buf);
        const float2 *trow = (a.flags & ROW_TRANS)
                                 ? (a.trans_b ? a.trans_b[line / a.nx] : a.trans) + (size_t)(line % a.nx) * N
                                 : nullptr;
        if (!load && store && lane == 0) tma_wait_read<NBUF - 1>();  // the store of line k-NBUF left buf
        if constexpr (NBUF == 2) {
            // two buffers: the next line goes into the buffer of line k-1 as soon as
            // that line's store has read it, so it loads while line k is transformed
            if (load && lane == 0 && k + 1 < nmine) {
                if (store) tma_wait_read<0>();
                issue(k + 1);
            }
        }
        float2 v[E];
        if (load) {
            const bool got = mbar_wait_bounded(&bar[s], (uint32_t)((k / NBUF) & 1), kWaitLimit);
            if (__any_sync(0xffffffffu, !got)) {
                ok = false;
                break;
            }
#pragma unroll
            for (int e = 0; e < E; ++e) v[e] = buf[t + T * e];
        } else {
#pragma unroll
            for (int e = 0; e < E; ++e) v[e] = make_float2(1.f, 0.f);
        }
        if (a.flags & ROW_INV) fft_line<P, -1, 0, true>(v, t, ad, tw);
        if (a.flags & ROW_TRANS) {
#pragma unroll
            for (int e = 0; e < E; ++e) v[e] = c_mul(v[e], __ldg(trow + t + T * e));
        }
        if (a.flags & ROW_FWD) fft_line<P, +1, 0, true>(v, t, ad, tw);
        if (a.scale != 1.0f) {
#pragma unroll
            for (int e = 0; e < E; ++e) v[e] = c_scale(v[e], a.scale);
        }
        if (a.flags & ROW_ACCUM) {
            double *acc = a.accum + (size_t)line * N;
#pragma unroll
            for (int e = 0; e < E; ++e)
                acc[t + T * e] += a.accum_w * ((double)v[e].x * v[e].x + (double)v[e].y * v[e].y);
        }
        if (store) {
            __syncwarp();  // every lane is done reading the slot
#pragma unroll
            for (int e = 0; e < E; ++e) buf[t + T * e] = v[e];
            fence_proxy_async();
            __syncwarp();
            if (lane == 0) {
                bulk_store(a.out + (size_t)unit * LPW * N, slot, (uint32_t)Cfg::UNIT);
                tma_commit();
            }
        }
        if constexpr (NBUF == 3) {
            if (load && lane == 0 && k + NBUF - 1 < nmine) {
                if (store) tma_wait_read<1>();  // the store of line k-1 has left its buffer
                issue(k + NBUF - 1);            // into buffer (k + 2) % 3
            }
        }
        __syncwarp();
    }
    if (lane == 0) {
        if (store) tma_wait_all();
        if (!ok) {
            if (a.err) atomicExch(a.err, 1);
            for (int j = k; j < issued; ++j)
                mbar_wait_bounded(&bar[j % NBUF], (uint32_t)((j / NBUF) & 1), kWaitLimit);
        }
    }
}

// ------------------------------------- two-stage row pass, 256 / 512 / 1024
// Row pass in the two-stage layouts (HalfWarpPlan256 / 512: each warp
// transforms two consecutive lines at a time, one per half-warp; WarpPlan1024x2:
// one line per warp): two register stages and a single exchange per transform
// (the three-stage warp layout needs two).  Lines arrive in units of one or two
// by 1D bulk copy into a private two-slot ring per warp; the next unit is
// requested once the previous unit's store has read its slot.  The stage-1
// twiddle table is formed in shared memory at start-up.
template <class P_> struct RowTwoCfg {
    using P = P_;
    // CTAs per SM: 3 at 32 elements per thread (registers), 5 at 16
    static constexpr int N = P::N, W = 4, THREADS = 32 * W, NBUF = 2, MINB = P::E >= 32 ? 3 : 5;
    static constexpr int LPW = 32 / P::T;  // lines per warp: 2 (half-warp lines) or 1
    static constexpr int R0 = P::radix(0), R1 = P::radix(1);
    static constexpr size_t LINE = sizeof(float2) * N, SLOT = LPW * LINE;
    static constexpr uint32_t ALIGN = (uint32_t)LINE;  // each line's exchange space is line-aligned
    // stage 1 table [r][k], k < R0, in shared memory: every r < R1, or rows 0
    // and 1 when the plan forms the powers w^r in registers (CW), or none when
    // the plan reads the table from the host-built twiddle buffer (GTW)
    static constexpr int TW = P::GTW ? 0 : (P::CW ? 2 : R1) * R0;
    static_assert(P::NSTAGE == 2 && R0 * R1 == N && (P::T == 16 || P::T == 32), "two-stage warp-owned lines");
    static constexpr size_t OFF_TW = (size_t)W * NBUF * SLOT;
    static constexpr size_t OFF_BAR = OFF_TW + sizeof(float2) * TW;
    static constexpr size_t SMEM = OFF_BAR + sizeof(uint64_t) * W * NBUF + ALIGN;
};

template <class P>
__global__ void __launch_bounds__(RowTwoCfg<P>::THREADS, RowTwoCfg<P>::MINB) row_two_kernel(RowArgs a) {
    using Cfg = RowTwoCfg<P>;
    constexpr int N = Cfg::N, E = P::E, T = P::T, NBUF = Cfg::NBUF, W = Cfg::W, LPW = Cfg::LPW, R0 = Cfg::R0;
    constexpr uint32_t AL = Cfg::ALIGN;
    extern __shared__ unsigned char smraw[];
    unsigned char *base = smraw + ((AL - (smem_u32(smraw) & (AL - 1u))) & (AL - 1u));
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, h = lane / T, t = lane % T;
    float2 *ring = reinterpret_cast<float2 *>(base) + (size_t)warp * NBUF * LPW * N;
    float2 *tw = reinterpret_cast<float2 *>(base + Cfg::OFF_TW);
    uint64_t *bar = reinterpret_cast<uint64_t *>(base + Cfg::OFF_BAR) + warp * NBUF;
    for (int i = threadIdx.x; i < Cfg::TW; i += Cfg::THREADS) {
        float sn, cn;
        sincospif((float)(2 * (i / R0) * (i % R0)) / (float)N, &sn, &cn);  // exp(2 pi i r k / N), [r][k]
        tw[i] = make_float2(cn, sn);
    }
    const float2 *twp = P::GTW ? a.tw + P::GTW_OFF : tw;
    if (lane == 0) {
        for (int s = 0; s < NBUF; ++s) mbar_init(&bar[s], 1);
        mbar_fence_init();
    }
    __syncthreads();  // the only CTA barrier: tables and barriers are ready
    const bool load = (a.flags & ROW_LOAD) != 0, store = !(a.flags & ROW_NOSTORE);
    const int npairs = a.nlines / LPW;  // units of LPW consecutive lines
    const int G = gridDim.x * W, gw = blockIdx.x * W + warp;
    const int nmine = gw < npairs ? (npairs - gw + G - 1) / G : 0;
    int issued = 0;
    auto issue = [&](int k) {  // lane 0 only
        const int pair = gw + k * G, s = k % NBUF;
        fence_proxy_async();
        mbar_arrive_expect_tx(&bar[s], (uint32_t)Cfg::SLOT);
        bulk_load(ring + (size_t)s * LPW * N, a.in + (size_t)pair * LPW * N, (uint32_t)Cfg::SLOT, &bar[s]);
        issued = k + 1;
    };
    if (load && lane == 0 && nmine > 0) issue(0);
    int k = 0;
    bool ok = true;
    for (; k < nmine; ++k) {
        const int pair = gw + k * G, s = k % NBUF, line = LPW * pair + h;
        float2 *slot = ring + (size_t)s * LPW * N;
        float2 *buf = slot + (size_t)h * N;
        const RowXorLin<P> ad{smem_u32(buf)};
        const float2 *trow = (a.flags & ROW_TRANS)
                                 ? (a.trans_b ? a.trans_b[line / a.nx] : a.trans) + (size_t)(line % a.nx) * N
                                 : nullptr;
        if (!load && store && lane == 0) tma_wait_read<NBUF - 1>();  // the store of pair k-2 left the slot
        if (load && lane == 0 && k + 1 < nmine) {
            if (store) tma_wait_read<0>();  // the store of pair k-1 has read the other slot
            issue(k + 1);
        }
        float2 v[E];
        if (load) {
            const bool got = mbar_wait_bounded(&bar[s], (uint32_t)((k / NBUF) & 1), kWaitLimit);
            if (__any_sync(0xffffffffu, !got)) {
                ok = false;
                break;
            }
#pragma unroll
            for (int e = 0; e < E; ++e) v[e] = buf[t + T * e];
        } else {
#pragma unroll
            for (int e = 0; e < E; ++e) v[e] = make_float2(1.f, 0.f);
        }
        if (a.flags & ROW_INV) fft_line_tab<P, -1>(v, t, ad, twp);
        if (a.flags & ROW_TRANS) {
#pragma unroll
            for (int e = 0; e < E; ++e) v[e] = c_mul(v[e], __ldg(trow + t + T * e));
        }
        if (a.flags & ROW_FWD) fft_line_tab<P, +1>(v, t, ad, twp);
        if (a.scale != 1.0f) {
#pragma unroll
            for (int e = 0; e < E; ++e) v[e] = c_scale(v[e], a.scale);
        }
        if (a.flags & ROW_ACCUM) {
            double *acc = a.accum + (size_t)line * N;
#pragma unroll
            for (int e = 0; e < E; ++e)
                acc[t + T * e] += a.accum_w * ((double)v[e].x * v[e].x + (double)v[e].y * v[e].y);
        }
        if (store) {
            __syncwarp();  // every lane is done reading the slot
#pragma unroll
            for (int e = 0; e < E; ++e) buf[t + T * e] = v[e];
            fence_proxy_async();
            __syncwarp();
            if (lane == 0) {
                bulk_store(a.out + (size_t)pair * LPW * N, slot, (uint32_t)Cfg::SLOT);
                tma_commit();
            }
        }
        __syncwarp();
    }
    if (lane == 0) {
        if (store) tma_wait_all();
        if (!ok) {
            if (a.err) atomicExch(a.err, 1);
            for (int j = k; j < issued; ++j)
                mbar_wait_bounded(&bar[j % NBUF], (uint32_t)((j / NBUF) & 1), kWaitLimit);
        }
    }
}

template <class P> static cudaError_t row_two_launch(const RowArgs &a, cudaStream_t s, int nsm) {
    using Cfg = RowTwoCfg<P>;
    static KernelSetup ks;
    int per_sm = 0;
    {
        cudaError_t e = ks.get(row_two_kernel<P>, Cfg::THREADS, Cfg::SMEM, false, &per_sm);
        if (e != cudaSuccess) return e;
    }
    const int nwarps = (a.nlines / Cfg::LPW + Cfg::W - 1) / Cfg::W;
    int grid = nsm * per_sm < nwarps ? nsm * per_sm : nwarps;
    if (grid < 1) grid = 1;
    row_two_kernel<P><<<grid, Cfg::THREADS, Cfg::SMEM, s>>>(a);
    return cudaGetLastError();
}

// ------------------------------------------ row pass, warp-pair lines, 2048
// Lines of 2048 points held by a warp pair (64 threads x 32 elements) in three
// register stages (WarpPairPlan2048); the two exchanges synchronise the pair on
// a named barrier.  Each pair streams its lines through a private two-slot ring
// of 16 KB-aligned line buffers (xor-linear exchange addresses) filled and
// drained by 1D bulk copies; its first lane issues the copies.  Three pairs per
// CTA, two CTAs per SM.  A wait that times out is voted over the pair, so both
// warps leave together.
struct RowPairCfg {
    using P = WarpPairPlan2048;
    static constexpr int N = P::N, W = 6, PAIRS = W / 2, THREADS = 32 * W, NBUF = 2, MINB = 2;
    static constexpr uint32_t LINE = sizeof(float2) * N;  // 16 KB, also the line alignment
    static constexpr int TW = plan_cwb_size<P>();
    static constexpr size_t OFF_BAR = ((sizeof(float2) * TW + 15) / 16) * 16;
    static constexpr size_t HEADER = OFF_BAR + sizeof(uint64_t) * PAIRS * NBUF;
    static constexpr size_t RING = (size_t)PAIRS * NBUF * LINE;
    static constexpr size_t SMEM = LINE + RING;  // the header, then the ring from the next line boundary
    static_assert(HEADER < LINE && P::T == 64, "warp-pair lines");
};

__global__ void __launch_bounds__(RowPairCfg::THREADS, RowPairCfg::MINB) row_pair_kernel(RowArgs a) {
    using Cfg = RowPairCfg;
    using P = Cfg::P;
    constexpr int N = Cfg::N, E = P::E, T = P::T, NBUF = Cfg::NBUF, PAIRS = Cfg::PAIRS;
    constexpr uint32_t LINE = Cfg::LINE;
    extern __shared__ unsigned char smraw[];
    const uint32_t sbase = smem_u32(smraw);
    const uint32_t ring0 = (sbase + (uint32_t)Cfg::HEADER + LINE - 1u) & ~(LINE - 1u);
    if (ring0 + (uint32_t)Cfg::RING > sbase + (uint32_t)Cfg::SMEM) {  // uniform over the CTA
        if (threadIdx.x == 0 && a.err) atomicExch(a.err, 2);         // layout error, not a timeout
        return;
    }
    float2 *tw = reinterpret_cast<float2 *>(smraw);
    uint64_t *barall = reinterpret_cast<uint64_t *>(smraw + Cfg::OFF_BAR);
#pragma unroll
    for (int st = 1; st < P::NSTAGE; ++st) {  // bases exp(2 pi i k / (NS R)), k < NS
        const int R = P::radix(st), NS = plan_span<P>(st), off = plan_cwb_offset<P>(st);
        for (int i = threadIdx.x; i < NS; i += Cfg::THREADS) {
            float sn, cn;
            sincospif((float)(2 * i) / (float)(NS * R), &sn, &cn);
            tw[off + i] = make_float2(cn, sn);
        }
    }
    if (threadIdx.x == 0) {
        for (int i = 0; i < PAIRS * NBUF; ++i) mbar_init(&barall[i], 1);
        mbar_fence_init();
    }
    __syncthreads();  // the only CTA-wide barrier
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, pr = warp >> 1;
    const int t = 32 * (warp & 1) + lane;
    const bool leader = t == 0;
    const uint32_t barid = 1u + (uint32_t)pr;
    auto pairsync = [&]() { bar_group(barid, 64); };
    uint64_t *bar = barall + pr * NBUF;
    const uint32_t ring = ring0 + (uint32_t)(pr * NBUF) * LINE;
    const bool load = (a.flags & ROW_LOAD) != 0, store = !(a.flags & ROW_NOSTORE);
    const int G = gridDim.x * PAIRS, gp = blockIdx.x * PAIRS + pr;
    const int nmine = gp < a.nlines ? (a.nlines - gp + G - 1) / G : 0;
    int issued = 0;
    auto issue = [&](int k) {  // the pair's first thread only
        const int line = gp + k * G, s = k % NBUF;
        fence_proxy_async();
        mbar_arrive_expect_tx(&bar[s], LINE);
        bulk_load(smraw + (ring + (uint32_t)s * LINE - sbase), a.in + (size_t)line * N, LINE, &bar[s]);
        issued = k + 1;
    };
    if (load && leader && nmine > 0) issue(0);
    int k = 0;
    bool ok = true;
    for (; k < nmine; ++k) {
        const int line = gp + k * G, s = k % NBUF;
        float2 *buf = reinterpret_cast<float2 *>(smraw + (ring + (uint32_t)s * LINE - sbase));
        const RowXorLin<P> ad{ring + (uint32_t)s * LINE};
        const float2 *trow = (a.flags & ROW_TRANS)
                                 ? (a.trans_b ? a.trans_b[line / a.nx] : a.trans) + (size_t)(line % a.nx) * N
                                 : nullptr;
        if (!load && store && leader) tma_wait_read<NBUF - 1>();  // the store of line k-2 left the slot
        if (load && leader && k + 1 < nmine) {
            if (store) tma_wait_read<0>();  // the store of line k-1 has read the other slot
            issue(k + 1);
        }
        float2 v[E];
        if (load) {
            const bool got = mbar_wait_bounded(&bar[s], (uint32_t)((k / NBUF) & 1), kWaitLimit);
            if (bar_group_or(barid, 64, !got)) {
                ok = false;
                break;
            }
#pragma unroll
            for (int e = 0; e < E; ++e) v[e] = buf[t + T * e];
        } else {
#pragma unroll
            for (int e = 0; e < E; ++e) v[e] = make_float2(1.f, 0.f);
        }
        if (a.flags & ROW_INV) fft_line_cwb<P, -1>(v, t, ad, tw, pairsync);
        if (a.flags & ROW_TRANS) {
#pragma unroll
            for (int e = 0; e < E; ++e) v[e] = c_mul(v[e], __ldg(trow + t + T * e));
        }
        if (a.flags & ROW_FWD) fft_line_cwb<P, +1>(v, t, ad, tw, pairsync);
        if (a.scale != 1.0f) {
#pragma unroll
            for (int e = 0; e < E; ++e) v[e] = c_scale(v[e], a.scale);
        }
        if (a.flags & ROW_ACCUM) {
            double *acc = a.accum + (size_t)line * N;
#pragma unroll
            for (int e = 0; e < E; ++e)
                acc[t + T * e] += a.accum_w * ((double)v[e].x * v[e].x + (double)v[e].y * v[e].y);
        }
        pairsync();  // both warps are done reading the slot (and, without a load, the old store left it)
        if (store) {
#pragma unroll
            for (int e = 0; e < E; ++e) buf[t + T * e] = v[e];
            fence_proxy_async();
            pairsync();
            if (leader) {
                bulk_store(a.out + (size_t)line * N, buf, LINE);
                tma_commit();
            }
        }
    }
    if (leader) {
        if (store) tma_wait_all();
        if (!ok) {
            if (a.err) atomicExch(a.err, 1);
            for (int j = k; j < issued; ++j)
                mbar_wait_bounded(&bar[j % NBUF], (uint32_t)((j / NBUF) & 1), kWaitLimit);
        }
    }
}

static cudaError_t row_pair_launch(const RowArgs &a, cudaStream_t s, int nsm) {
    using Cfg = RowPairCfg;
    static KernelSetup ks;
    int per_sm = 0;
    {
        cudaError_t e = ks.get(row_pair_kernel, Cfg::THREADS, Cfg::SMEM, true, &per_sm);
        if (e != cudaSuccess) return e;
    }
    const int ncta = (a.nlines + Cfg::PAIRS - 1) / Cfg::PAIRS;
    int grid = nsm * per_sm < ncta ? nsm * per_sm : ncta;
    if (grid < 1) grid = 1;
    row_pair_kernel<<<grid, Cfg::THREADS, Cfg::SMEM, s>>>(a);
    return cudaGetLastError();
}

// ------------------------------------------------------------ set-up kernels
__global__ void probe_table_kernel(int nx, int ny, const double *kxd, const double *kyd,
                                   double s_in, double s_out, double lam, double df, double cs,
                                   double scale, float2 *apchi) {
    const int iy = blockIdx.x * blockDim.x + threadIdx.x;
    const int ix = blockIdx.y;
    if (iy >= ny || ix >= nx) return;
    const double s = __dadd_rn(__dmul_rn(kxd[ix], kxd[ix]), __dmul_rn(kyd[iy], kyd[iy]));
    float2 out = make_float2(0.f, 0.f);
    if (s >= s_in && s <= s_out) {
        // chi = pi (lambda df s + Cs lambda^3 s^2 / 2)   (MSProject.cs:511-514)
        const double chi = 3.14159265358979323846 * (lam * df * s + 0.5 * cs * lam * lam * lam * s * s);
        double sn, cn;
        sincos(chi, &sn, &cn);
        out = make_float2((float)(cn * scale), (float)(-sn * scale));
    }
    apchi[(size_t)ix * ny + iy] = out;
}

__global__ void probe_shift_kernel(int nx, int ny, int nb, const double *fxy, float2 *ex,
                                   float2 *ey) {
    const int b = blockIdx.y;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nb) return;
    if (i < nx) {
        const int si = i < nx / 2 ? i : i - nx;
        double p = (double)si * fxy[2 * b];
        p -= rint(p);
        double sn, cn;
        sincospi(2.0 * p, &sn, &cn);
        ex[(size_t)b * nx + i] = make_float2((float)cn, (float)sn);
    }
    if (i < ny) {
        const int sj = i < ny / 2 ? i : i - ny;
        double p = (double)sj * fxy[2 * b + 1];
        p -= rint(p);
        double sn, cn;
        sincospi(2.0 * p, &sn, &cn);
        ey[(size_t)b * ny + i] = make_float2((float)cn, (float)sn);
    }
}

__global__ void detector_mask_kernel(int nx, int ny, const double *kxd, const double *kyd, int ndet,
                                     const double *kin2, const double *kout2, uint8_t *mask) {
    const int iy = blockIdx.x * blockDim.x + threadIdx.x;
    const int ix = blockIdx.y;
    if (iy >= ny || ix >= nx) return;
    const double s = __dadd_rn(__dmul_rn(kxd[ix], kxd[ix]), __dmul_rn(kyd[iy], kyd[iy]));
    unsigned bits = 0;
    for (int d = 0; d < ndet; ++d)
        if (s <= kout2[d] && s >= kin2[d]) bits |= 1u << d;
    mask[(size_t)ix * ny + iy] = (uint8_t)bits;
}

__global__ void ctf_table_kernel(int nx, int ny, const float *kx2, const float *ky2, const float *kx,
                                 const float *ky, CtfParams p, float2 *ctf) {
    const int iy = blockIdx.x * blockDim.x + threadIdx.x;
    const int ix = blockIdx.y;
    if (iy >= ny || ix >= nx) return;
    const float k2 = __fadd_rn(kx2[ix], ky2[iy]);
    float2 out = make_float2(0.f, 0.f);
    if (k2 <= p.k2obj) {
        const double q = (double)k2;
        double w = 0.5 * p.cs * p.lam * p.lam * q - p.df;
        if (p.dfa2 != 0.0 || p.dfa3 != 0.0) {
            const double phi = atan2((double)ky[iy], (double)kx[ix]);
            w += p.dfa2 * sin(2.0 * (phi - p.dfa2phi)) +
                 2.0 * p.dfa3 * p.lam * sqrt(q) * sin(3.0 * (phi - p.dfa3phi)) / 3.0;
        }
        const double chi = 3.14159265358979323846 * p.lam * q * w;
        double sn, cn;
        sincos(chi, &sn, &cn);
        out = make_float2((float)cn * p.scale, (float)-sn * p.scale);
    }
    ctf[(size_t)ix * ny + iy] = out;
}

__global__ void tilt_wave_kernel(int nx, int ny, const float *xpos, const float *ypos, const float *q,
                                 float2 *out) {
    const int iy = blockIdx.x * blockDim.x + threadIdx.x;
    const int ix = blockIdx.y, b = blockIdx.z;
    if (iy >= ny || ix >= nx) return;
    const float s = __fadd_rn(__fmul_rn(q[2 * b], xpos[ix]), __fmul_rn(q[2 * b + 1], ypos[iy]));
    const double t = 2.0 * (double)3.14159265f * (double)s;
    double sn, cn;
    sincos(t, &sn, &cn);
    out[((size_t)b * nx + ix) * ny + iy] = make_float2((float)cn, (float)sn);
}

// Transmission function t = exp(i sigma V) of every pixel (mulslice.cpp:414-421).
// The phase carries FP64-grade accuracy in float-float arithmetic (FP64
// instructions run at a small fraction of the FP32 rate on this GPU and bound
// an FP64 version of this elementwise kernel): sigma = s_hi + s_lo, the product
// s_hi V kept exactly as p + e (fma), then a Cody-Waite reduction by 2 pi split
// into three floats (C1 = 6.28125 has 8 significant bits, so k C1 is exact for
// |k| < 2^16), the low parts added last.  The reduced phase in [-pi, pi] then
// goes to the single-precision sincos.  Elementwise, so the band-limiting
// transforms that follow run on the fast row / column kernels.
__global__ void transmission_phase_kernel(const float *__restrict__ v, float s_hi, float s_lo, size_t n,
                                          float2 *__restrict__ t) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const float x = v[i];
        const float p = s_hi * x;
        const float e = fmaf(s_hi, x, -p) + s_lo * x;  // sigma x = p + e to about 48 bits
        const float k = rintf(p * 0.15915494309189535f);
        float r = fmaf(-k, 6.28125f, p);
        r = fmaf(-k, 1.9353071693331003e-3f, r);
        r += e;
        r = fmaf(-k, 1.0253131677018246e-11f, r);
        float sn, cn;
        sincosf(r, &sn, &cn);
        t[i] = make_float2(cn, sn);
    }
}

// Self-test of the bounded waits: an mbarrier that nothing ever arrives on is
// polled `polls` times; the wait gives up, the kernel raises *err and returns.
__global__ void wait_timeout_kernel(int *err, uint32_t polls) {
    __shared__ uint64_t bar;
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        mbar_fence_init();
    }
    __syncthreads();
    const bool got = mbar_wait_bounded(&bar, 0u, polls);
    if (__syncthreads_or(!got) && threadIdx.x == 0) atomicExch(err, 1);
}

__global__ void detector_finalize_kernel(int nb, int ntile, int ndet, const double *partial,
                                         double scale, double *out, int out_stride) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nb * ndet) return;
    const int b = i / ndet, d = i % ndet;
    double s = 0.0;
    for (int t = 0; t < ntile; ++t) s += partial[((size_t)b * ntile + t) * ndet + d];
    out[(size_t)b * out_stride + d] = s * scale;
}

// Frozen-phonon STEM: image j * np + p is configuration j of probe p; the
// configurations' sums are added to the running total one after another.
__global__ void detector_accumulate_kernel(int nconf, int np, int ntile, int ndet, const double *partial,
                                           double scale, double *out, int out_stride) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= np * ndet) return;
    const int p = i / ndet, d = i % ndet;
    double v = out[(size_t)p * out_stride + d];
    for (int j = 0; j < nconf; ++j) {
        const double *q = partial + (size_t)(j * np + p) * ntile * ndet + d;
        double s = 0.0;
        for (int t = 0; t < ntile; ++t) s += q[(size_t)t * ndet];
        v += s * scale;
    }
    out[(size_t)p * out_stride + d] = v;
}

// ----------------------------------------------------------------- dispatch
template <int N> static cudaError_t row_launch(const RowArgs &a, cudaStream_t s, int nsm) {
    static KernelSetup ks;
    int blocks_per_sm = 0;
    {
        cudaError_t e = ks.get(row_pass_kernel<N>, RowCfg<N>::THREADS, RowCfg<N>::SMEM, false, &blocks_per_sm);
        if (e != cudaSuccess) return e;
    }
    const int ngroups = (a.nlines + RowCfg<N>::LPB - 1) / RowCfg<N>::LPB;
    int grid = nsm * blocks_per_sm;
    if (grid > ngroups) grid = ngroups;
    if (grid < 1) grid = 1;
    dim3 block(Plan<N>::T, RowCfg<N>::LPB);
    row_pass_kernel<N><<<grid, block, RowCfg<N>::SMEM, s>>>(a);
    return cudaGetLastError();
}

template <int N> static cudaError_t col_launch(const ColArgs &a, cudaStream_t s, int nsm) {
    static KernelSetup ks;
    int blocks_per_sm = 0;
    {
        cudaError_t e = ks.get(col_pass_kernel<N>, ColCfg<N>::THREADS, ColCfg<N>::SMEM, false, &blocks_per_sm);
        if (e != cudaSuccess) return e;
    }
    const int ntiles = a.batch * (a.ny / ColCfg<N>::C);
    int grid = nsm * blocks_per_sm;
    if (grid > ntiles) grid = ntiles;
    if (grid < 1) grid = 1;
    col_pass_kernel<N><<<grid, ColCfg<N>::THREADS, ColCfg<N>::SMEM, s>>>(a);
    return cudaGetLastError();
}


typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *,
                                  const cuuint64_t *, const cuuint64_t *, const cuuint32_t *,
                                  const cuuint32_t *, CUtensorMapInterleave, CUtensorMapSwizzle,
                                  CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static EncodeTiledFn lookup_encode_fn() {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
        return (EncodeTiledFn)p;
    cudaGetLastError();
    return nullptr;
}

// The driver entry point is process-wide; the static's initialisation is thread-safe.
static EncodeTiledFn encode_fn() {
    static const EncodeTiledFn fn = lookup_encode_fn();
    return fn;
}

// The TMA kernel needs one buffer for load and store (in place) at a 16-byte
// aligned address; other calls take the register-only kernel.
static bool tma_eligible(const ColArgs &a) {
    if (!a.out || ((uintptr_t)a.out & 15u)) return false;
    if ((a.flags & COL_LOAD) && a.in != a.out) return false;
    if (!(a.flags & (COL_LOAD | COL_STORE))) return false;
    return encode_fn() != nullptr;
}

template <class PL, int MINB> static cudaError_t col_tma_launch_v(const ColArgs &a, cudaStream_t s, int nsm) {
    using Cfg = ColTmaCfg<PL>;
    constexpr int N = PL::N;
    static KernelSetup ks;
    int per_sm = 0;
    {
        cudaError_t e = ks.get(col_tma_kernel<PL, MINB>, Cfg::THREADS, Cfg::SMEM, false, &per_sm);
        if (e != cudaSuccess) return e;
    }
    CUtensorMap map;
    const cuuint64_t gdim[2] = {(cuuint64_t)a.ny, (cuuint64_t)a.batch * N};
    const cuuint64_t gstride[1] = {(cuuint64_t)a.ny * sizeof(float2)};
    const cuuint32_t box[2] = {(cuuint32_t)Cfg::C, (cuuint32_t)Cfg::BOXR};
    const cuuint32_t estride[2] = {1, 1};
    CUresult r = encode_fn()(&map, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 2, (void *)a.out, gdim, gstride, box,
                             estride, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                             CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return cudaErrorInvalidValue;
    const int ntiles = a.batch * (a.ny / Cfg::C);
    int grid = nsm * per_sm < ntiles ? nsm * per_sm : ntiles;
    if (grid < 1) grid = 1;
    col_tma_kernel<PL, MINB><<<grid, Cfg::THREADS, Cfg::SMEM, s>>>(map, a);
    return cudaGetLastError();
}

template <class L> static cudaError_t col_half_launch(const ColArgs &a, cudaStream_t s, int nsm) {
    using Cfg = ColHalfCfg<L>;
    static KernelSetup ks;
    int per_sm = 0;
    {
        cudaError_t e = ks.get(col_half_kernel<L>, Cfg::THREADS, Cfg::SMEM, true, &per_sm);
        if (e != cudaSuccess) return e;
    }
    CUtensorMap map;
    const cuuint64_t gdim[2] = {(cuuint64_t)a.ny, (cuuint64_t)a.batch * Cfg::N};
    const cuuint64_t gstride[1] = {(cuuint64_t)a.ny * sizeof(float2)};
    const cuuint32_t box[2] = {(cuuint32_t)Cfg::C, (cuuint32_t)Cfg::BOXR};
    const cuuint32_t estride[2] = {1, 1};
    CUresult r = encode_fn()(&map, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 2, (void *)a.out, gdim, gstride, box,
                             estride, CU_TENSOR_MAP_INTERLEAVE_NONE, L::SWZ,
                             CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return cudaErrorInvalidValue;
    const int ngroups = (a.batch * (a.ny / Cfg::C) + Cfg::G - 1) / Cfg::G;
    int grid = nsm * per_sm < ngroups ? nsm * per_sm : ngroups;
    if (grid < 1) grid = 1;
    col_half_kernel<L><<<grid, Cfg::THREADS, Cfg::SMEM, s>>>(map, a);
    return cudaGetLastError();
}
// The column pass the slice loop takes at side n (0: col_tma_kernel): every
// pass that loads the wave and starts with the forward transform, with or
// without the inverse (a scan's last slice detects only), so all detector
// passes of a scan write partials per 4 columns.
static int col_half_side(int n, const ColArgs &a) {
    if (!(a.flags & COL_LOAD) || !(a.flags & COL_FWD) || (a.flags & COL_PROBE)) return 0;
    if (n == 256 && a.ny % ColHalfL256::C == 0) return 256;
    if (n == 512 && a.ny % ColHalfL512::C == 0) return 512;
    if (n == 1024 && a.ny % ColPairL1024::C == 0) return 1024;
    return 0;
}
template <int N> static cudaError_t col_tma_launch(const ColArgs &a, cudaStream_t s, int nsm) {
    return col_tma_launch_v<ColPlan<N>, ColPlan<N>::MINB>(a, s, nsm);
}


static bool row_tma_eligible(const RowArgs &a) {
    if (!a.out || ((uintptr_t)a.out & 15u)) return false;
    if ((a.flags & ROW_LOAD) && a.in != a.out) return false;
    if (a.flags & ROW_GENT) return false;
    return encode_fn() != nullptr;
}

template <int N, int TH, int MINB>
static cudaError_t row_tma_launch_v(const RowArgs &a, cudaStream_t s, int nsm) {
    using Cfg = RowTmaCfg<N, TH>;
    static KernelSetup ks;
    int per_sm = 0;
    {
        cudaError_t e = ks.get(row_tma_kernel<N, TH, MINB>, Cfg::THREADS, Cfg::SMEM, false, &per_sm);
        if (e != cudaSuccess) return e;
    }
    if (a.nlines % Cfg::L) return cudaErrorInvalidValue;
    CUtensorMap map;
    const cuuint64_t gdim[3] = {(cuuint64_t)Cfg::BX, (cuuint64_t)Cfg::NBX, (cuuint64_t)a.nlines};
    const cuuint64_t gstride[2] = {(cuuint64_t)Cfg::BX * sizeof(float2), (cuuint64_t)N * sizeof(float2)};
    const cuuint32_t box[3] = {(cuuint32_t)Cfg::BX, (cuuint32_t)Cfg::NBX, (cuuint32_t)Cfg::L};
    const cuuint32_t estride[3] = {1, 1, 1};
    CUresult r = encode_fn()(&map, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 3, (void *)a.out, gdim, gstride, box,
                             estride, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                             CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return cudaErrorInvalidValue;
    const int ntiles = a.nlines / Cfg::L;
    int grid = nsm * per_sm < ntiles ? nsm * per_sm : ntiles;
    if (grid < 1) grid = 1;
    row_tma_kernel<N, TH, MINB><<<grid, Cfg::THREADS, Cfg::SMEM, s>>>(map, a);
    return cudaGetLastError();
}

// 128-thread CTAs, as many per SM as registers and shared memory allow (six
// for 8-element lines): timing the 512 case, more independent CTAs beat wider
// ones because every exchange of a line transform is a CTA-wide barrier.
template <int N> static cudaError_t row_tma_launch(const RowArgs &a, cudaStream_t s, int nsm) {
    return row_tma_launch_v<N, 128, (Plan<N>::E <= 8 ? 6 : 4)>(a, s, nsm);
}


template <int N> static cudaError_t row_warp_launch(const RowArgs &a, cudaStream_t s, int nsm) {
    using Cfg = RowWarpCfg<N>;
    static KernelSetup ks;
    int per_sm = 0;
    {
        cudaError_t e = ks.get(row_warp_kernel<N>, Cfg::THREADS, Cfg::SMEM, false, &per_sm);
        if (e != cudaSuccess) return e;
    }
    const int nwarps = (a.nlines / Cfg::LPW + Cfg::W - 1) / Cfg::W;
    int grid = nsm * per_sm < nwarps ? nsm * per_sm : nwarps;
    if (grid < 1) grid = 1;
    row_warp_kernel<N><<<grid, Cfg::THREADS, Cfg::SMEM, s>>>(a);
    return cudaGetLastError();
}

// Warp-owned lines for the sides whose plan fits 32 threads per line.
static bool row_warp_eligible(int ny, const RowArgs &a) {
    if (ny != 256 && ny != 384 && ny != 512 && ny != 768 && ny != 1024 && ny != 2048) return false;
    if (a.flags & ROW_GENT) return false;
    if (((uintptr_t)a.out & 15u) || ((a.flags & ROW_LOAD) && ((uintptr_t)a.in & 15u))) return false;
    return true;
}

// ------------------------------------------------------------- schedules
// Which kernel family each side's row and column passes take, per device: the
// fast family (the warp-owned / two-stage / warp-pair kernels), the TMA-tiled
// kernels, or the register-only kernels.  Set by the autotuner
// (msl_autotune) or by hand (msl_set_schedule); all families compute the same
// transforms (the pass-family tests check each against the oracle).
namespace {
std::atomic<int> g_sched_row[kMaxDevices][8];
std::atomic<int> g_sched_col[kMaxDevices][8];

int side_slot(int n) {
    switch (n) {
        case 64: return 0;
        case 128: return 1;
        case 256: return 2;
        case 384: return 3;
        case 512: return 4;
        case 768: return 5;
        case 1024: return 6;
        case 2048: return 7;
        default: return -1;
    }
}

int current_device() {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
        cudaGetLastError();
        return 0;
    }
    return dev;
}

int sched_row(int n) {
    const int k = side_slot(n);
    return k < 0 ? FAM_FAST : g_sched_row[current_device()][k].load(std::memory_order_relaxed);
}
int sched_col(int n) {
    const int k = side_slot(n);
    return k < 0 ? FAM_FAST : g_sched_col[current_device()][k].load(std::memory_order_relaxed);
}
}  // namespace

bool set_schedule(int n, int row_family, int col_family) {
    const int k = side_slot(n);
    if (k < 0 || row_family < 0 || row_family > FAM_TC || col_family < 0 || col_family > FAM_TC) return false;
    if ((row_family == FAM_TC || col_family == FAM_TC) && !tc_side(n)) return false;
    const int dev = current_device();
    g_sched_row[dev][k].store(row_family);
    g_sched_col[dev][k].store(col_family);
    return true;
}

bool get_schedule(int n, int *row_family, int *col_family) {
    if (side_slot(n) < 0) return false;
    *row_family = sched_row(n);
    *col_family = sched_col(n);
    return true;
}

bool plan_supported(int n) {
    switch (n) {
#define X(N) case N:
        MSL_FOR_EACH_SIDE(X)
#undef X
        return true;
        default: return false;
    }
}

int plan_col_c(int n) {
    switch (n) {
#define X(N) case N: return Plan<N>::col_c;
        MSL_FOR_EACH_SIDE(X)
#undef X
        default: return 0;
    }
}

static bool col_tc_eligible(int nx, const ColArgs &a);

int plan_col_c_launch(int n, const ColArgs &a) {
    const int fam0 = sched_col(n);
    if (fam0 == FAM_TC) {
        // the slice loop's column passes (loaded, forward) run on the tensor cores in tiles of 8 columns
        ColArgs f = a;
        f.flags = COL_LOAD | COL_FWD | COL_PROP;
        f.in = f.out;
        if (col_tc_eligible(n, f)) return tc_col_tile();
    }
    const int fam = fam0 == FAM_TC ? FAM_FAST : fam0;
    if (fam != FAM_REG && tma_eligible(a)) {
        // the slice loop's column pass (load, forward, inverse) on two-stage
        // columns writes detector partials per 4 columns
        ColArgs f = a;
        f.flags = (f.flags | COL_LOAD | COL_FWD) & ~COL_PROBE;
        if (fam == FAM_FAST && col_half_side(n, f)) return 4;
        switch (n) {
#define X(N) case N: return ColPlan<N>::col_c;
            MSL_FOR_EACH_SIDE(X)
#undef X
            default: return 0;
        }
    }
    return plan_col_c(n);
}

template <int N> static void twiddles_fill(float2 *out) {
    using P = Plan<N>;
    for (int s = 1; s < P::NSTAGE; ++s) {
        const int R = P::radix(s), NS = plan_span<P>(s), off = plan_tw_offset<P>(s);
        for (int r = 0; r < R; ++r)
            for (int k = 0; k < NS; ++k) {
                // exp(+2 pi i r k / (NS R)), argument reduced exactly in integers
                const long m = ((long)r * k) % ((long)NS * R);
                const double ang = 2.0 * 3.14159265358979323846 * (double)m / (double)(NS * R);
                out[off + r * NS + k] = make_float2((float)cos(ang), (float)sin(ang));
            }
    }
}

template <int N> static void twiddles_for(std::vector<float2> &out) {
    out.assign(plan_tw_size<Plan<N>>() > 0 ? plan_tw_size<Plan<N>>() : 1, make_float2(0.f, 0.f));
    twiddles_fill<N>(out.data());
}

void plan_twiddles(int n, std::vector<float2> &out) {
    switch (n) {
#define X(N) case N: twiddles_for<N>(out); break;
        MSL_FOR_EACH_SIDE(X)
#undef X
        default: out.clear();
    }
    const int extra = row_two_twiddles_size(n);
    if (extra > (int)out.size()) {
        out.resize(extra);
        append_row_two_twiddles(n, out.data());
    }
}

int plan_twiddles_into(int n, float2 *out, int cap) {
    int size = 0;
    switch (n) {
#define X(N) case N: size = plan_tw_size<Plan<N>>() > 0 ? plan_tw_size<Plan<N>>() : 1; break;
        MSL_FOR_EACH_SIDE(X)
#undef X
        default: return -1;
    }
    if (row_two_twiddles_size(n) > size) size = row_two_twiddles_size(n);
    if (size > cap) return -1;
    for (int i = 0; i < size; ++i) out[i] = make_float2(0.f, 0.f);
    switch (n) {
#define X(N) case N: twiddles_fill<N>(out); break;
        MSL_FOR_EACH_SIDE(X)
#undef X
        default: return -1;
    }
    append_row_two_twiddles(n, out);
    return size;
}

int row_two_twiddles_size(int n) {
    return n == WarpPlan1024x2::N && WarpPlan1024x2::GTW ? WarpPlan1024x2::GTW_OFF + 32 * 32 : 0;
}

void append_row_two_twiddles(int n, float2 *tables) {
    if (!row_two_twiddles_size(n)) return;
    // the two-stage 1024 row plan's stage-1 table [r][k] = exp(2 pi i r k / 1024),
    // r, k < 32, after Plan<1024>'s own tables (read through L1 by the row kernel)
    using P = WarpPlan1024x2;
    for (int r = 0; r < 32; ++r)
        for (int k = 0; k < 32; ++k) {
            const double ph = 2.0 * 3.14159265358979323846 * (double)((r * k) % 1024) / 1024.0;
            tables[(size_t)P::GTW_OFF + r * 32 + k] = make_float2((float)cos(ph), (float)sin(ph));
        }
}

// The slice loop's row pass (load, inverse, * t, forward, store) on the tensor cores.
static bool row_tc_eligible(int ny, const RowArgs &a) {
    const int need = ROW_LOAD | ROW_INV | ROW_TRANS | ROW_FWD;
    return tc_side(ny) && (a.flags & ~need) == 0 && a.flags == need && a.in == a.out && a.scale == 1.0f &&
           a.nlines % tc_col_tile() == 0 && a.nx % tc_col_tile() == 0;
}
// The slice loop's column pass (load, forward, propagator, [detect], [inverse, store]).
static bool col_tc_eligible(int nx, const ColArgs &a) {
    const int base = COL_LOAD | COL_FWD | COL_PROP;
    const int rest = a.flags & ~(base | COL_DETECT);
    if (!tc_side(nx) || (a.flags & base) != base || a.in != a.out || a.prop_b || a.k2_b) return false;
    if (rest != 0 && rest != (COL_INV | COL_STORE)) return false;
    return a.ny % tc_col_tile() == 0;
}
static TcPassArgs tc_row_args(int ny, const RowArgs &a) {
    TcPassArgs t = {};
    t.data = a.out;
    t.nlines = a.nlines;
    t.nx = a.nx;
    t.ny = ny;
    t.cols = 0;
    t.dir1 = -1;
    t.dir2 = +1;
    t.second = 1;
    t.mode = TC_MODE_TRANS;
    t.trans = a.trans;
    t.trans_b = a.trans_b;
    t.err = a.err;
    return t;
}
static TcPassArgs tc_col_args(int nx, const ColArgs &a) {
    TcPassArgs t = {};
    t.data = a.out;
    t.nlines = a.batch * a.ny;
    t.nx = nx;
    t.ny = a.ny;
    t.cols = 1;
    t.dir1 = +1;
    t.dir2 = -1;
    t.second = (a.flags & COL_INV) ? 1 : 0;
    t.mode = TC_MODE_PROP;
    t.px = a.px;
    t.py = a.py;
    t.kx2 = a.kx2;
    t.ky2 = a.ky2;
    t.k2max = a.k2max;
    if (a.flags & COL_DETECT) {
        t.detmask = a.detmask;
        t.ndet = a.ndet;
        t.partial = a.partial;
    }
    t.err = a.err;
    return t;
}

cudaError_t launch_row_pass(int ny, const RowArgs &a, cudaStream_t s, int nsm, int64_t *launches) {
    const int fam0 = sched_row(ny);
    if (fam0 == FAM_TC && row_tc_eligible(ny, a)) return launch_tc_pass(tc_row_args(ny, a), s, nsm, launches);
    ++*launches;
    const int fam = fam0 == FAM_TC ? FAM_FAST : fam0;
    if (fam == FAM_FAST && row_warp_eligible(ny, a)) {
        switch (ny) {
            case 256:
                if (a.nlines % 2 == 0 && !(((uintptr_t)a.out | (uintptr_t)a.in) & 15u))
                    return row_two_launch<HalfWarpPlan256>(a, s, nsm);
                return row_warp_launch<256>(a, s, nsm);
            case 384:  // half-warp lines: in pairs
                if (a.nlines % 2 == 0) return row_warp_launch<384>(a, s, nsm);
                break;
            case 768: return row_warp_launch<768>(a, s, nsm);
            case 512:
                if (a.nlines % 2 == 0 && !(((uintptr_t)a.out | (uintptr_t)a.in) & 15u))
                    return row_two_launch<HalfWarpPlan512>(a, s, nsm);
                return row_warp_launch<512>(a, s, nsm);
            case 1024: return row_two_launch<WarpPlan1024x2>(a, s, nsm);
            case 2048: return row_pair_launch(a, s, nsm);
            default: break;
        }
    }
    if (fam != FAM_REG && row_tma_eligible(a)) {
        switch (ny) {
#define X(N) case N: return row_tma_launch<N>(a, s, nsm);
            MSL_FOR_EACH_SIDE(X)
#undef X
            default: return cudaErrorInvalidValue;
        }
    }
    switch (ny) {
#define X(N) case N: return row_launch<N>(a, s, nsm);
        MSL_FOR_EACH_SIDE(X)
#undef X
        default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_col_pass(int nx, const ColArgs &a, cudaStream_t s, int nsm, int64_t *launches) {
    const int fam0 = sched_col(nx);
    if (fam0 == FAM_TC && col_tc_eligible(nx, a)) return launch_tc_pass(tc_col_args(nx, a), s, nsm, launches);
    ++*launches;
    const int fam = fam0 == FAM_TC ? FAM_FAST : fam0;
    if (fam != FAM_REG && tma_eligible(a)) {
        // the slice loop's passes at 256, 512 and 1024: two-stage columns
        switch (fam == FAM_FAST ? col_half_side(nx, a) : 0) {
            case 256: return col_half_launch<ColHalfL256>(a, s, nsm);
            case 512: return col_half_launch<ColHalfL512>(a, s, nsm);
            case 1024: return col_half_launch<ColPairL1024>(a, s, nsm);
            default: break;
        }
        switch (nx) {
#define X(N) case N: return col_tma_launch<N>(a, s, nsm);
            MSL_FOR_EACH_SIDE(X)
#undef X
            default: return cudaErrorInvalidValue;
        }
    }
    switch (nx) {
#define X(N) case N: return col_launch<N>(a, s, nsm);
        MSL_FOR_EACH_SIDE(X)
#undef X
        default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_probe_table(int nx, int ny, const double *kxd, const double *kyd, double s_in,
                               double s_out, double lam, double df, double cs, double scale,
                               float2 *apchi, cudaStream_t s, int64_t *launches) {
    ++*launches;
    dim3 grid((ny + 255) / 256, nx);
    probe_table_kernel<<<grid, 256, 0, s>>>(nx, ny, kxd, kyd, s_in, s_out, lam, df, cs, scale, apchi);
    return cudaGetLastError();
}

cudaError_t launch_probe_shifts(int nx, int ny, int nb, const double *fxy, float2 *ex, float2 *ey,
                                cudaStream_t s, int64_t *launches) {
    ++*launches;
    const int n = nx > ny ? nx : ny;
    dim3 grid((n + 255) / 256, nb);
    probe_shift_kernel<<<grid, 256, 0, s>>>(nx, ny, nb, fxy, ex, ey);
    return cudaGetLastError();
}

cudaError_t launch_detector_mask(int nx, int ny, const double *kxd, const double *kyd, int ndet,
                                 const double *kin2, const double *kout2, uint8_t *mask,
                                 cudaStream_t s, int64_t *launches) {
    ++*launches;
    dim3 grid((ny + 255) / 256, nx);
    detector_mask_kernel<<<grid, 256, 0, s>>>(nx, ny, kxd, kyd, ndet, kin2, kout2, mask);
    return cudaGetLastError();
}

cudaError_t launch_ctf_table(int nx, int ny, const float *kx2, const float *ky2, const float *kx,
                             const float *ky, const CtfParams &p, float2 *ctf, cudaStream_t s,
                             int64_t *launches) {
    ++*launches;
    dim3 grid((ny + 255) / 256, nx);
    ctf_table_kernel<<<grid, 256, 0, s>>>(nx, ny, kx2, ky2, kx, ky, p, ctf);
    return cudaGetLastError();
}

cudaError_t launch_tilt_waves(int nx, int ny, int nb, const float *xpos, const float *ypos,
                              const float *q, float2 *out, cudaStream_t s, int64_t *launches) {
    ++*launches;
    dim3 grid((ny + 255) / 256, nx, nb);
    tilt_wave_kernel<<<grid, 256, 0, s>>>(nx, ny, xpos, ypos, q, out);
    return cudaGetLastError();
}

cudaError_t launch_transmission_phase(const float *v, double scale, size_t n, float2 *t, int nsm, cudaStream_t s,
                                      int64_t *launches) {
    ++*launches;
    const float s_hi = (float)scale, s_lo = (float)(scale - (double)s_hi);
    size_t blocks = (n + 255) / 256;
    const size_t cap = (size_t)nsm * 16;
    if (blocks > cap) blocks = cap;
    if (blocks < 1) blocks = 1;
    transmission_phase_kernel<<<(unsigned)blocks, 256, 0, s>>>(v, s_hi, s_lo, n, t);
    return cudaGetLastError();
}

cudaError_t launch_wait_timeout(int *err, uint32_t polls, cudaStream_t s, int64_t *launches) {
    ++*launches;
    wait_timeout_kernel<<<1, 64, 0, s>>>(err, polls);
    return cudaGetLastError();
}

cudaError_t launch_detector_accumulate(int nconf, int np, int ntile, int ndet, const double *partial,
                                       double scale, double *out, int out_stride, cudaStream_t s,
                                       int64_t *launches) {
    ++*launches;
    const int n = np * ndet;
    detector_accumulate_kernel<<<(n + 127) / 128, 128, 0, s>>>(nconf, np, ntile, ndet, partial, scale, out,
                                                               out_stride);
    return cudaGetLastError();
}

cudaError_t launch_detector_finalize(int nb, int ntile, int ndet, const double *partial,
                                     double scale, double *out, int out_stride, cudaStream_t s,
                                     int64_t *launches) {
    ++*launches;
    const int n = nb * ndet;
    detector_finalize_kernel<<<(n + 255) / 256, 256, 0, s>>>(nb, ntile, ndet, partial, scale, out,
                                                            out_stride);
    return cudaGetLastError();
}

}  // namespace msl
