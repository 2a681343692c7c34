// Line DFTs of the slice loop as dense contractions on the tensor cores.
//
// A line of N = 16 N2 points (N = 256: N2 = 16; N = 512: N2 = 32) is
// transformed in two contraction stages (the four-step factorisation):
//   D1 (input order L1: row (l, n2) holds x[N2 n1 + n2] over n1)
//      stage 1: DFT16 over n1            -> row (l, n2), columns k1
//      twiddle W_N^(n2 k1), transpose    -> row (l, k1), columns n2
//      stage 2: DFT_N2 over n2           -> row (l, k1) holds X[k1 + 16 k2] over k2   (order L2)
//   D2 (input order L2: row (l, na) holds x[na + 16 nb] over nb)
//      stage A: DFT_N2 over nb           -> row (l, na), columns kb
//      twiddle W_N^(na kb), transpose    -> row (l, kb), columns na
//      stage B: DFT16 over na            -> row (l, kb) holds X[N2 ka + kb] over ka    (order L1)
// so a pass (transform, pointwise work in order L2, transform back) starts and
// ends in order L1 with no data movement between its two transforms.  Every
// stage is D = A B^T on tcgen05 (M = 128 rows per MMA, FP32 accumulator in
// tensor memory) with complex numbers as real pairs -- B is the real form
// [[Wr, -Wi], [Wi, Wr]] of the DFT matrix -- and FP32 accuracy won back by
// split-bf16 products: each operand is hi + lo (hi = bf16(x), lo = bf16(x - hi))
// and A is packed [hi | lo] along K against B1 = [Bhi | Bhi] and B2 = [Blo | 0],
// so D = Ahi Bhi + Alo Bhi + Ahi Blo (the lo lo term, 2^-16 relative, dropped).
// Only the + sign matrices are held: a transform of sign -1 is computed as
// conj(DFT+(conj(x))), the conjugations being sign flips where the operand is
// written and the result read, so a CTA fits in half the shared memory and two
// run per SM.
// The row pass (ifft_y, * t, fft_y) and the column pass (fft_x, propagator and
// band limit, [detector sums], ifft_x) of msl_passes.cu take this path when
// the side's schedule is MSL_FAM_TC; twiddles, pointwise factors and detector
// sums stay FP32 / FP64 as in the FP32 passes.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "msl_internal.h"
#include "msl_tc.cuh"

namespace msl {

namespace {

constexpr int kTcLines = 8;      // lines per tile
constexpr int kTcThreads = 256;  // 8 warps
constexpr uint32_t kTcWait = 1u << 22;

template <int N> struct TcGeom {
    static constexpr int N2 = N / 16;
    static constexpr int R1 = kTcLines * N2;     // rows of the DFT16 stages (128 or 256)
    static constexpr int MT1 = R1 / 128;         // their 128-row MMA tiles
    static constexpr int KR2 = 2 * N2;           // real K of the DFT_N2 stages (32 or 64)
    static constexpr int ATOM2 = KR2 == 32 ? 1 : 2;  // 128-byte K atoms of a DFT_N2 A row ([hi|lo])
    // shared memory (1024-byte aligned tiles)
    static constexpr size_t A1 = (size_t)R1 * 128;              // DFT16 stage A operand: [hi 32 | lo 32]
    static constexpr size_t A2 = (size_t)128 * 128 * ATOM2;     // DFT_N2 stage A operand
    static constexpr size_t B16 = 32 * 128;                     // one DFT16 B tile (32 rows)
    static constexpr size_t BN2 = (size_t)KR2 * 128;            // one DFT_N2 B tile per K atom
    static constexpr size_t OFF_A1 = 0;
    static constexpr size_t OFF_A2 = OFF_A1 + A1;
    // B tiles of the + sign only: [B1|B2] for DFT16, [B1|B2][atom] for DFT_N2 (a
    // transform of sign -1 runs as conj(DFT+(conj(x))): the conjugations are sign
    // flips in the epilogues)
    static constexpr size_t OFF_B16 = OFF_A2 + A2;
    static constexpr size_t OFF_BN2 = OFF_B16 + 2 * B16;
    static constexpr size_t OFF_TW = OFF_BN2 + 2 * ATOM2 * BN2;       // W_N^m, m < N
    static constexpr size_t OFF_RED = OFF_TW + sizeof(float2) * N;
    static constexpr size_t SMEM = OFF_RED + sizeof(double) * 8 * 8 + 1024;
    // CTAs per SM: registers (launch bounds) and shared memory allow four at 256, two at 512
    static constexpr int MINB = N == 256 ? 4 : 2;
    static_assert(MINB * (SMEM + 2048) <= 233472, "MINB CTAs fit an SM's shared memory");
    // the staging of the tile's output lines reuses the DFT_N2 operand (free by then)
    static constexpr size_t OFF_OUT = OFF_A2;
    static_assert(A2 >= sizeof(float2) * kTcLines * N, "output staging fits the DFT_N2 operand");
};

// A complex value (re, im) as split-bf16 K pairs: (hi re, hi im) at K positions
// k, k + 1 (k even) and (lo re, lo im) at kr + k, kr + k + 1 -- one 4-byte store
// each.  K runs over [hi | lo] halves of kr; complex inputs are interleaved
// (re, im) along K, and the B operands are built with the same order.
__device__ __forceinline__ void split_store2(unsigned char *tile, int row, int k, int kr, float re, float im) {
    const __nv_bfloat16 hr = __float2bfloat16_rn(re), hi_ = __float2bfloat16_rn(im);
    const __nv_bfloat16 lr = __float2bfloat16_rn(re - __bfloat162float(hr));
    const __nv_bfloat16 li = __float2bfloat16_rn(im - __bfloat162float(hi_));
    const int kh = k, kl = kr + k;
    *(__nv_bfloat162 *)(tile + (kh >> 6) * 128 * 128 + tc::sw128_offset(row, kh & 63)) = __halves2bfloat162(hr, hi_);
    *(__nv_bfloat162 *)(tile + (kl >> 6) * 128 * 128 + tc::sw128_offset(row, kl & 63)) = __halves2bfloat162(lr, li);
}

// Real form of the L-point DFT of sign dir: row (k, part), column (n, part),
// part 0 real 1 imaginary; columns [0, L) real inputs, [L, 2L) imaginary.
__device__ __forceinline__ float dft_real(int L, int dir, int row, int col) {
    const int k = row % L, pr = row / L, n = col % L, pc = col / L;
    float s, c;
    sincospif((float)(2 * ((k * n) % L)) / (float)L, &s, &c);
    s *= (float)dir;
    // out_re = sum c x_re - s x_im ; out_im = sum s x_re + c x_im
    if (pr == 0) return pc == 0 ? c : -s;
    return pc == 0 ? s : c;
}

// B1 = [hi | hi], B2 = [lo | 0] of the real DFT matrix (rows = 2L outputs, K = 2L inputs
// in the order (n, part) interleaved, as split_store2 writes A), K packed
// [hi part | lo part] over atoms of 64; tile t = atom index.
__device__ void build_b(unsigned char *b1, unsigned char *b2, int L, int dir, size_t atom_bytes) {
    const int R = 2 * L;
    for (int i = threadIdx.x; i < R * R; i += blockDim.x) {
        const int row = i / R, col = i % R;
        const float w = dft_real(L, dir, row, col);
        const __nv_bfloat16 hi = __float2bfloat16_rn(w);
        const __nv_bfloat16 lo = __float2bfloat16_rn(w - __bfloat162float(hi));
        const int kh = 2 * (col % L) + col / L, kl = R + kh;  // K order (n, part) interleaved
        *(__nv_bfloat16 *)(b1 + (kh >> 6) * atom_bytes + tc::sw128_offset(row, kh & 63)) = hi;
        *(__nv_bfloat16 *)(b1 + (kl >> 6) * atom_bytes + tc::sw128_offset(row, kl & 63)) = hi;
        *(__nv_bfloat16 *)(b2 + (kh >> 6) * atom_bytes + tc::sw128_offset(row, kh & 63)) = lo;
        *(__nv_bfloat16 *)(b2 + (kl >> 6) * atom_bytes + tc::sw128_offset(row, kl & 63)) = __float2bfloat16_rn(0.f);
    }
}

// One stage: D[tmem] = A (rows m0.., `atoms` K atoms) x (B1 + B2)^T.  Thread 0 issues.
__device__ __forceinline__ void stage_mma(uint32_t tmem, const unsigned char *a, size_t a_atom_bytes,
                                          const unsigned char *b1, const unsigned char *b2, size_t b_atom_bytes,
                                          int atoms, int n, bool skip_b2_last) {
    const uint32_t idesc = tc::idesc_bf16(128, n);
    bool first = true;
    for (int at = 0; at < atoms; ++at)
        for (int which = 0; which < 2; ++which) {
            if (which == 1 && skip_b2_last && at == atoms - 1) continue;  // B2's lo half is zero there
            const unsigned char *b = which == 0 ? b1 : b2;
#pragma unroll
            for (int kk = 0; kk < 4; ++kk) {
                tc::mma_bf16(tmem, tc::desc_sw128(smem_u32(a + at * a_atom_bytes) + kk * 32),
                             tc::desc_sw128(smem_u32(b + at * b_atom_bytes) + kk * 32), idesc, first ? 0u : 1u);
                first = false;
            }
        }
}

}  // namespace

template <int N>
__global__ void __launch_bounds__(kTcThreads, TcGeom<N>::MINB) tc_pass_kernel(TcPassArgs a) {
    using G = TcGeom<N>;
    constexpr int N2 = G::N2;
    extern __shared__ __align__(1024) unsigned char smraw[];
    unsigned char *base = (unsigned char *)(((uintptr_t)smraw + 1023) & ~(uintptr_t)1023);
    unsigned char *A1 = base + G::OFF_A1, *A2 = base + G::OFF_A2;
    float2 *twn = (float2 *)(base + G::OFF_TW);
    float2 *stage = (float2 *)(base + G::OFF_OUT);
    double *red = (double *)(base + G::OFF_RED);
    __shared__ uint64_t bar;
    __shared__ uint32_t tmem_base;
    __shared__ int failed;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    // conjugations that turn the + sign transforms into the - sign ones
    const float c1 = a.dir1 > 0 ? 1.f : -1.f, c2 = a.dir2 > 0 ? 1.f : -1.f;
    // constant operands: DFT16 and DFT_N2 of the + sign
    build_b(base + G::OFF_B16, base + G::OFF_B16 + G::B16, 16, 1, G::B16);
    build_b(base + G::OFF_BN2, base + G::OFF_BN2 + (size_t)G::ATOM2 * G::BN2, N2, 1, G::BN2);
    const unsigned char *b16_1 = base + G::OFF_B16, *b16_2 = base + G::OFF_B16 + G::B16;
    const unsigned char *bn2_1 = base + G::OFF_BN2, *bn2_2 = base + G::OFF_BN2 + (size_t)G::ATOM2 * G::BN2;
    for (int m = tid; m < N; m += kTcThreads) {
        float s, c;
        sincospif((float)(2 * m) / (float)N, &s, &c);
        twn[m] = make_float2(c, s);  // W_N^m for the + sign
    }
    if (warp == 0) tc::tmem_alloc(&tmem_base, 64);
    if (tid == 0) {
        mbar_init(&bar, 1);
        mbar_fence_init();
        failed = 0;
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = tmem_base;
    uint32_t phase = 0;
    auto run = [&](const unsigned char *A, size_t a_atom, const unsigned char *b1, const unsigned char *b2,
                   size_t b_atom, int atoms, int n, int mtiles, size_t a_mtile_bytes) {
        fence_proxy_async();
        __syncthreads();
        if (tid == 0 && !failed) {
            tc::fence_after_sync();
            for (int mt = 0; mt < mtiles; ++mt)
                stage_mma(tmem + (uint32_t)(mt * n), A + mt * a_mtile_bytes, a_atom, b1, b2, b_atom, atoms, n,
                          atoms == 2);
            tc::mma_commit(&bar);
        }
        if (!mbar_wait_bounded(&bar, phase, kTcWait)) failed = 1;
        phase ^= 1u;
        tc::fence_after_sync();
        __syncthreads();
    };
    const bool cols = a.cols != 0;
    const int per_img = cols ? a.ny : a.nx;      // lines per image
    const int ntiles = a.nlines / kTcLines;
    for (int tile = blockIdx.x; tile < ntiles && !failed; tile += gridDim.x) {
        const int line0 = tile * kTcLines, img = line0 / per_img, lin0 = line0 % per_img;
        // element (l, n) of the tile in global memory
        auto gaddr = [&](int l, int n) -> float2 * {
            return cols ? a.data + ((size_t)img * a.nx + n) * a.ny + lin0 + l
                        : a.data + ((size_t)img * a.nx + lin0 + l) * a.ny + n;
        };
        // ---- load in order L1 into the DFT16 operand: row (l, n2), K n1 (re) / 16 + n1 (im);
        // all of a thread's loads are issued before its shared-memory stores
        constexpr int PER = kTcLines * N / kTcThreads, CH = 8;  // in chunks of 8 (registers)
        static_assert(PER % CH == 0, "load chunks");
#pragma unroll 1
        for (int j0 = 0; j0 < PER; j0 += CH) {
            float2 xin[CH];
#pragma unroll
            for (int j = 0; j < CH; ++j) {
                const int i = tid + (j0 + j) * kTcThreads;
                const int l = cols ? i % kTcLines : i / N, n = cols ? i / kTcLines : i % N;
                xin[j] = *gaddr(l, n);
            }
#pragma unroll
            for (int j = 0; j < CH; ++j) {
                const int i = tid + (j0 + j) * kTcThreads;
                const int l = cols ? i % kTcLines : i / N, n = cols ? i / kTcLines : i % N;
                const int row = l * N2 + n % N2, k = n / N2;
                unsigned char *t = A1 + (row >> 7) * 128 * 128;
                split_store2(t, row & 127, 2 * k, 32, xin[j].x, c1 * xin[j].y);
            }
        }
        // ---------------- transform 1 (D1, sign dir1: the + transform of the input conjugated by c1)
        run(A1, 128 * 128, b16_1, b16_2, G::B16, 1, 32, G::MT1, 128 * 128);
        if (failed) break;
        // stage-1 epilogue: row (l, n2) -> twiddle W^(n2 k1) -> row (l, k1), K n2.
        // Two 128-row tiles (N = 512): warps 4-7 take the second; one tile (N = 256):
        // warps 0-3 take k1 0..7 and warps 4-7 k1 8..15 of the same rows.
        {
            const int wq = warp & 3, hi = warp >> 2;
            const int r = (G::MT1 == 2 ? hi * 128 : 0) + 32 * wq + lane;
            const uint32_t tcol = (uint32_t)(G::MT1 == 2 ? hi * 32 : 0);
            const int c0 = G::MT1 == 2 ? 0 : hi * 8, nk = G::MT1 == 2 ? 16 : 8;
            const int l = r / N2, n2 = r % N2;
            const uint32_t lanes = (uint32_t)(32 * wq) << 16;
            for (int c = 0; c < nk; c += 8) {
                float re[8], im[8];
                tc::tmem_ld8(tmem + lanes + tcol + (uint32_t)(c0 + c), re);        // k1 real parts
                tc::tmem_ld8(tmem + lanes + tcol + (uint32_t)(16 + c0 + c), im);   // k1 imaginary parts
#pragma unroll
                for (int j = 0; j < 8; ++j) {
                    const int k1 = c0 + c + j;
                    const float2 tw = twn[(n2 * k1) % N];
                    const float xr = re[j] * tw.x - im[j] * tw.y, xi = re[j] * tw.y + im[j] * tw.x;
                    const int row2 = l * 16 + k1;
                    split_store2(A2, row2, 2 * n2, G::KR2, xr, xi);
                }
            }
        }
        run(A2, 128 * 128, bn2_1, bn2_2, G::BN2, G::ATOM2, G::KR2, 1, 0);
        if (failed) break;
        // stage-2 epilogue (order L2): row (l, k1) holds X[k1 + 16 k2]; pointwise work, then
        // the same row becomes D2's stage-A operand (K = k2)
        const bool second = a.second != 0;
        {
            const int wq = warp & 3, half = warp >> 2;
            const int row = 32 * wq + lane, l = row / 16, k1 = row % 16;
            const int line = lin0 + l;
            constexpr int H = N2 / 2;  // k2 handled by this thread: [half H, half H + H)
            float re[H], im[H];
            for (int c = 0; c < H; c += 16) {
                float v[16], w[16];
                const int cc = half * H + c;
                tc::tmem_ld16(tmem + ((uint32_t)(32 * wq) << 16) + (uint32_t)cc, v);
                tc::tmem_ld16(tmem + ((uint32_t)(32 * wq) << 16) + (uint32_t)(N2 + cc), w);
#pragma unroll
                for (int j = 0; j < 16 && c + j < H; ++j) {
                    re[c + j] = v[j];
                    im[c + j] = w[j];
                }
            }
            double acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
#pragma unroll
            for (int c = 0; c < H; ++c) {
                const int k2 = half * H + c, n = k1 + 16 * k2;   // element index along the line
                float2 x = make_float2(re[c], c1 * im[c]);
                if (a.mode == TC_MODE_TRANS) {
                    // row lines: line = ix, n = iy
                    const float2 *tr = a.trans_b ? a.trans_b[img] : a.trans;
                    const float2 t = __ldg(tr + (size_t)line * N + n);
                    x = make_float2(x.x * t.x - x.y * t.y, x.x * t.y + x.y * t.x);
                } else if (a.mode == TC_MODE_PROP) {
                    // column lines: line = iy, n = ix
                    const float k2v = a.kx2[n] + a.ky2[line];
                    if (k2v < a.k2max) {
                        const float2 p1 = __ldg(a.py + line), p2 = __ldg(a.px + n);
                        const float2 y = make_float2(x.x * p1.x - x.y * p1.y, x.x * p1.y + x.y * p1.x);
                        x = make_float2(y.x * p2.x - y.y * p2.y, y.x * p2.y + y.y * p2.x);
                    } else {
                        x = make_float2(0.f, 0.f);
                    }
                    if (a.detmask) {
                        const uint32_t m = a.detmask[(size_t)n * a.ny + line];
                        const double p = (double)x.x * x.x + (double)x.y * x.y;
#pragma unroll
                        for (int d = 0; d < 8; ++d)
                            if (m & (1u << d)) acc[d] += p;
                    }
                }
                if (second) {
                    split_store2(A2, row, 2 * k2, G::KR2, x.x, c2 * x.y);
                }
            }
            if (a.detmask) {
                // sums over the tile's 8 columns: warp, then the 8 warps in order
                for (int d = 0; d < a.ndet; ++d) {
                    double s = acc[d];
#pragma unroll
                    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
                    if (lane == 0) red[warp * 8 + d] = s;
                }
                __syncthreads();
                if (tid < a.ndet) {
                    double s = 0.0;
                    for (int w = 0; w < 8; ++w) s += red[w * 8 + tid];
                    a.partial[((size_t)img * (a.ny / kTcLines) + lin0 / kTcLines) * a.ndet + tid] = s;
                }
            }
        }
        if (!second) {
            __syncthreads();
            continue;
        }
        // ---------------- transform 2 (D2, sign dir2): stage A on A2 as written (conjugated by c2)
        run(A2, 128 * 128, bn2_1, bn2_2, G::BN2, G::ATOM2, G::KR2, 1, 0);
        if (failed) break;
        // stage-A epilogue: row (l, na), columns kb -> twiddle W^(na kb) -> row (l, kb), K na
        {
            const int wq = warp & 3, half = warp >> 2;
            const int row = 32 * wq + lane, l = row / 16, na = row % 16;
            constexpr int H = N2 / 2;
            float re[H], im[H];
            for (int c = 0; c < H; c += 16) {
                float v[16], w[16];
                const int cc = half * H + c;
                tc::tmem_ld16(tmem + ((uint32_t)(32 * wq) << 16) + (uint32_t)cc, v);
                tc::tmem_ld16(tmem + ((uint32_t)(32 * wq) << 16) + (uint32_t)(N2 + cc), w);
#pragma unroll
                for (int j = 0; j < 16 && c + j < H; ++j) {
                    re[c + j] = v[j];
                    im[c + j] = w[j];
                }
            }
#pragma unroll
            for (int c = 0; c < H; ++c) {
                const int kb = half * H + c;
                const float2 tw = twn[(na * kb) % N];
                const float xr = re[c] * tw.x - im[c] * tw.y, xi = re[c] * tw.y + im[c] * tw.x;
                const int row1 = l * N2 + kb;
                unsigned char *t = A1 + (row1 >> 7) * 128 * 128;
                split_store2(t, row1 & 127, 2 * na, 32, xr, xi);
            }
        }
        run(A1, 128 * 128, b16_1, b16_2, G::B16, 1, 32, G::MT1, 128 * 128);
        if (failed) break;
        // stage-B epilogue: row (l, kb) holds X[N2 ka + kb]: stage the tile, then store coalesced
        {
            const int wq = warp & 3, hi = warp >> 2;
            const int r = (G::MT1 == 2 ? hi * 128 : 0) + 32 * wq + lane;
            const uint32_t tcol = (uint32_t)(G::MT1 == 2 ? hi * 32 : 0);
            const int c0 = G::MT1 == 2 ? 0 : hi * 8, nk = G::MT1 == 2 ? 16 : 8;
            const int l = r / N2, kb = r % N2;
            const uint32_t lanes = (uint32_t)(32 * wq) << 16;
            for (int c = 0; c < nk; c += 8) {
                float re[8], im[8];
                tc::tmem_ld8(tmem + lanes + tcol + (uint32_t)(c0 + c), re);
                tc::tmem_ld8(tmem + lanes + tcol + (uint32_t)(16 + c0 + c), im);
#pragma unroll
                for (int j = 0; j < 8; ++j) stage[l * N + N2 * (c0 + c + j) + kb] = make_float2(re[j], c2 * im[j]);
            }
        }
        tc::fence_before_sync();
        __syncthreads();
        for (int i = tid; i < kTcLines * N; i += kTcThreads) {
            const int l = cols ? i % kTcLines : i / N, n = cols ? i / kTcLines : i % N;
            *gaddr(l, n) = stage[l * N + n];
        }
        __syncthreads();
    }
    if (failed && tid == 0 && a.err) atomicExch(a.err, 1);
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_free(tmem, 64);
}

template <int N> static cudaError_t tc_pass_launch(const TcPassArgs &a, cudaStream_t s, int nsm) {
    using G = TcGeom<N>;
    static KernelSetup ks;
    int per_sm = 0;
    cudaError_t e = ks.get(tc_pass_kernel<N>, kTcThreads, G::SMEM, true, &per_sm);
    if (e != cudaSuccess) return e;
    // G::MINB CTAs fit an SM by registers (launch bounds) and shared memory; the
    // occupancy query has answered fewer for this kernel, so the grid asks for
    // G::MINB per SM (a CTA that does not fit waits for a free slot)
    if (per_sm < G::MINB) per_sm = G::MINB;
    const int ntiles = a.nlines / kTcLines;
    int grid = nsm * per_sm < ntiles ? nsm * per_sm : ntiles;
    if (grid < 1) grid = 1;
    tc_pass_kernel<N><<<grid, kTcThreads, G::SMEM, s>>>(a);
    return cudaGetLastError();
}

bool tc_side(int n) { return n == 256 || n == 512; }

cudaError_t launch_tc_pass(const TcPassArgs &a, cudaStream_t s, int nsm, int64_t *launches) {
    if (a.nlines % kTcLines) return cudaErrorInvalidValue;
    ++*launches;
    switch (a.cols ? a.nx : a.ny) {
        case 256: return tc_pass_launch<256>(a, s, nsm);
        case 512: return tc_pass_launch<512>(a, s, nsm);
        default: return cudaErrorInvalidValue;
    }
}

int tc_col_tile() { return kTcLines; }

}  // namespace msl
