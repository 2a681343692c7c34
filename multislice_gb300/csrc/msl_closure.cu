// Learned coarse-slice closure: a complex-valued convolutional network that
// corrects an exit wave computed with 4x thicker slices toward the fine-slice
// result.  It has no counterpart in the reference; the reference's fine-slice
// loop (mulslice.cpp:706-739) is its fallback and the judge of its error.
//
// Network (complex channels, 3x3 taps, periodic boundaries as the wave itself):
//   x = psi / s                 (s = norm of psi / 256: its RMS on a 256^2 grid)
//   h1 = CReLU(conv(x; 1 -> C))
//   h2..h5 = CReLU(conv(h; C -> C))
//   d = conv(h5; C -> 1)
//   psi_out = psi + s d
// with CReLU applying max(0, .) to real and imaginary parts separately and
// C = 32.  A complex layer is held as a real layer over 2C channels (real parts
// then imaginary parts) whose weight blocks are [[Wr, -Wi], [Wi, Wr]].
//
// Kernels:
//   * conv_tc_kernel: the C -> C layers (K = 9 taps x 64 real channels,
//     N = 64) as an implicit GEMM on the tensor cores: 128 output pixels of an
//     image row per tile, one tcgen05.mma chain per tap from 128B-swizzled
//     shared-memory tiles, FP32 accumulator in tensor memory, bias + CReLU (or
//     the backward pass's ReLU mask) in the epilogue, bf16 activations out.
//     The same kernel computes the input gradient of these layers with the
//     flipped, transposed weights.
//   * conv_small_kernel: the 1 -> C and C -> 1 layers and the input gradient
//     of the last layer on the CUDA cores (FP32).
//   * dw_kernel: weight gradients on the CUDA cores, FP32 partial sums per
//     pixel block reduced in a fixed order (deterministic).
// Weights are kept as FP32 master copies (Adam) and used as bf16.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include <string.h>

#include <string>
#include <vector>

#include "../../include/msl.h"
#include "msl_internal.h"
#include "msl_tc.cuh"

namespace msl {
namespace closure {

constexpr int kC = 32;          // complex channels of the hidden layers
constexpr int kR = 2 * kC;      // real channels
constexpr int kLayers = 6;
constexpr int kTile = 128;      // output pixels per tensor-core tile
constexpr uint32_t kWait = 1u << 22;

// Parameter layout (FP32), per layer l with complex in/out counts (ci, co):
//   weights [9][co][ci][2] (re, im), then bias [co][2].
__host__ __device__ inline int layer_ci(int l) { return l == 0 ? 1 : kC; }
__host__ __device__ inline int layer_co(int l) { return l == kLayers - 1 ? 1 : kC; }
inline int layer_wsize(int l) { return 9 * layer_co(l) * layer_ci(l) * 2; }
inline int layer_size(int l) { return layer_wsize(l) + layer_co(l) * 2; }
inline int param_offset(int l) {
    int o = 0;
    for (int i = 0; i < l; ++i) o += layer_size(i);
    return o;
}
inline int param_count() { return param_offset(kLayers); }

// ------------------------------------------------------------------ helpers
__device__ __forceinline__ float bf(const __nv_bfloat16 v) { return __bfloat162float(v); }

// Real weight of the expanded layer: output real channel n, input real channel k.
__device__ __forceinline__ float expand_w(const float *wl, int co, int ci, int tap, int n, int k) {
    const int o = n % co, a = n / co, i = k % ci, b = k / ci;
    const float *w = wl + (((size_t)tap * co + o) * ci + i) * 2;
    if (a == b) return w[0];
    return a == 0 ? -w[1] : w[1];
}

// wt[tap][n][k] (bf16, K-major) = expanded real weights; transposed = the
// input-gradient form: wt[tap'][k][n] with tap' the mirrored tap.
__global__ void expand_kernel(const float *wl, int co, int ci, int transposed, __nv_bfloat16 *wt) {
    const int nr = 2 * co, kr = 2 * ci;
    const int total = 9 * nr * kr;
    for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < total; idx += gridDim.x * blockDim.x) {
        const int tap = idx / (nr * kr), rem = idx % (nr * kr);
        if (!transposed) {
            const int n = rem / kr, k = rem % kr;
            wt[idx] = __float2bfloat16_rn(expand_w(wl, co, ci, tap, n, k));
        } else {
            // output index [tap'][k][n]: rem = k * nr + n, source tap = 8 - tap'
            const int k = rem / nr, n = rem % nr;
            wt[idx] = __float2bfloat16_rn(expand_w(wl, co, ci, 8 - tap, n, k));
        }
    }
}

// dL/dtheta from dL/dW (real expanded, FP32 [9][2co][2ci]).
__global__ void contract_kernel(const float *dw, int co, int ci, float *g) {
    const int total = 9 * co * ci;
    const int nr = 2 * co, kr = 2 * ci;
    for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < total; idx += gridDim.x * blockDim.x) {
        const int tap = idx / (co * ci), o = (idx / ci) % co, i = idx % ci;
        const float *d = dw + (size_t)tap * nr * kr;
        const float rr = d[(size_t)o * kr + i], ii = d[(size_t)(co + o) * kr + ci + i];
        const float ri = d[(size_t)o * kr + ci + i], ir = d[(size_t)(co + o) * kr + i];
        g[(size_t)idx * 2] = rr + ii;        // dWr
        g[(size_t)idx * 2 + 1] = ir - ri;    // dWi
    }
}

// --------------------------------------------------- tensor-core C -> C layer
enum Epi { EPI_BIAS_RELU = 0, EPI_MASK = 1 };

constexpr size_t kWTile = 64 * 128;          // one tap's B tile: 64 rows x 128 bytes
constexpr size_t kATile = kTile * 128;       // 128 pixels x 128 bytes
constexpr size_t kConvSmem = 1024 + 9 * kWTile + 2 * kATile;

__global__ void __launch_bounds__(128) conv_tc_kernel(const __nv_bfloat16 *__restrict__ in,
                                                      const __nv_bfloat16 *__restrict__ wt,
                                                      const float *__restrict__ bias,
                                                      const __nv_bfloat16 *__restrict__ mask,
                                                      __nv_bfloat16 *__restrict__ out, int B, int H, int W, int epi,
                                                      int *err) {
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    unsigned char *base = (unsigned char *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    unsigned char *sw = base;                    // 9 x 8 KB
    unsigned char *sa = base + 9 * kWTile;       // 2 x 16 KB
    __shared__ uint64_t bar[2];
    __shared__ uint32_t tmem_base;
    __shared__ int failed;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    // all nine B tiles, resident for the whole kernel
    for (int i = tid; i < 9 * 64 * 8; i += 128) {
        const int tap = i / 512, r = (i / 8) % 64, c = i % 8;
        const uint4 v = *(const uint4 *)(wt + ((size_t)tap * 64 + r) * 64 + c * 8);
        *(uint4 *)(sw + tap * kWTile + tc::sw128_offset(r, c * 8)) = v;
    }
    if (warp == 0) tc::tmem_alloc(&tmem_base, 64);
    if (tid == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        mbar_fence_init();
        failed = 0;
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = tmem_base;
    const uint32_t idesc = tc::idesc_bf16(kTile, 64);
    const int xt = W / kTile, ntiles = B * H * xt;
    uint32_t u = 0;
    for (int t = blockIdx.x; t < ntiles && !failed; t += gridDim.x) {
        const int img = t / (H * xt), y = (t / xt) % H, x0 = (t % xt) * kTile;
        for (int tap = 0; tap < 9; ++tap, ++u) {
            const int s = u & 1;
            if (u >= 2 && !mbar_wait_bounded(&bar[s], ((u - 2) >> 1) & 1, kWait)) failed = 1;
            const int yy = (y + tap / 3 - 1 + H) % H, dx = tap % 3 - 1;
            const __nv_bfloat16 *row = in + ((size_t)img * H + yy) * W * 64;
            unsigned char *dst = sa + s * kATile;
            // the tap's 16 KB: every load of this thread issued before its stores
            constexpr int PER = kTile * 8 / 128;
            uint4 va[PER];
#pragma unroll
            for (int j = 0; j < PER; ++j) {
                const int i = tid + 128 * j, r = i >> 3, c = i & 7;
                const int xx = (x0 + r + dx + W) % W;
                va[j] = *(const uint4 *)(row + (size_t)xx * 64 + c * 8);
            }
#pragma unroll
            for (int j = 0; j < PER; ++j) {
                const int i = tid + 128 * j, r = i >> 3, c = i & 7;
                *(uint4 *)(dst + tc::sw128_offset(r, c * 8)) = va[j];
            }
            fence_proxy_async();
            __syncthreads();
            if (tid == 0 && !failed) {
                tc::fence_after_sync();
#pragma unroll
                for (int kk = 0; kk < 4; ++kk)
                    tc::mma_bf16(tmem, tc::desc_sw128(smem_u32(dst) + kk * 32),
                                 tc::desc_sw128(smem_u32(sw + tap * kWTile) + kk * 32), idesc,
                                 (tap > 0 || kk > 0) ? 1u : 0u);
                tc::mma_commit(&bar[s]);
            }
        }
        if (!mbar_wait_bounded(&bar[(u - 1) & 1], ((u - 1) >> 1) & 1, kWait)) failed = 1;
        tc::fence_after_sync();
        __syncthreads();
        if (failed) break;
        // epilogue: this thread's pixel (TMEM lane) and its 64 channels
        const int r = 32 * (warp & 3) + lane;
        const size_t pix = ((size_t)img * H + y) * W + x0 + r;
        const uint32_t lane_base = (uint32_t)(32 * (warp & 3)) << 16;
        __nv_bfloat16 *o = out + pix * 64;
#pragma unroll
        for (int c0 = 0; c0 < 64; c0 += 16) {
            float v[16];
            tc::tmem_ld16(tmem + lane_base + (uint32_t)c0, v);
            __align__(16) __nv_bfloat16 ob[16];
            if (epi == EPI_BIAS_RELU) {
#pragma unroll
                for (int j = 0; j < 16; ++j) {
                    // real channel n = c0 + j: the complex bias [o][2] holds (re, im) of channel n % 32
                    const int n = c0 + j;
                    ob[j] = __float2bfloat16_rn(fmaxf(v[j] + bias[(n & (kC - 1)) * 2 + (n >> 5)], 0.0f));
                }
            } else {
                const __nv_bfloat16 *m = mask + pix * 64 + c0;
#pragma unroll
                for (int j = 0; j < 16; ++j) ob[j] = __float2bfloat16_rn(bf(m[j]) > 0.0f ? v[j] : 0.0f);
            }
            *(uint4 *)(o + c0) = *(const uint4 *)ob;
            *(uint4 *)(o + c0 + 8) = *(const uint4 *)(ob + 8);
        }
        tc::fence_before_sync();
        __syncthreads();  // TMEM read out before the next tile's first MMA overwrites it
    }
    if (failed && tid == 0 && err) atomicExch(err, 1);
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_free(tmem, 64);
}

// ----------------------------------------------------- CUDA-core small layers
// First layer: x (complex64 [B][H][W], scaled by 1/s[b]) -> h1 = CReLU(conv + b)
// (bf16 [B][H][W][64]); the scaled input is also written as bf16 [B][H][W][2]
// for the weight gradient.
__global__ void first_layer_kernel(const float2 *__restrict__ psi, const float *__restrict__ inv_s,
                                   const float *__restrict__ wl, __nv_bfloat16 *__restrict__ xin,
                                   __nv_bfloat16 *__restrict__ h, int B, int H, int W) {
    __shared__ float w[9 * kC * 2 + kC * 2];
    for (int i = threadIdx.x; i < 9 * kC * 2 + kC * 2; i += blockDim.x) w[i] = wl[i];
    __syncthreads();
    const size_t npix = (size_t)B * H * W;
    for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < npix; p += (size_t)gridDim.x * blockDim.x) {
        const int b = (int)(p / ((size_t)H * W)), y = (int)((p / W) % H), x = (int)(p % W);
        const float sc = inv_s[b];
        float xr[9], xi[9];
#pragma unroll
        for (int tap = 0; tap < 9; ++tap) {
            const int yy = (y + tap / 3 - 1 + H) % H, xx = (x + tap % 3 - 1 + W) % W;
            const float2 v = psi[((size_t)b * H + yy) * W + xx];
            // the tensor-core layers see bf16 values: round the input the same way
            xr[tap] = __bfloat162float(__float2bfloat16_rn(v.x * sc));
            xi[tap] = __bfloat162float(__float2bfloat16_rn(v.y * sc));
        }
        xin[p * 2] = __float2bfloat16_rn(xr[4]);
        xin[p * 2 + 1] = __float2bfloat16_rn(xi[4]);
        __nv_bfloat16 *o = h + p * 64;
        for (int oc = 0; oc < kC; ++oc) {
            float ar = w[9 * kC * 2 + oc * 2], ai = w[9 * kC * 2 + oc * 2 + 1];
#pragma unroll
            for (int tap = 0; tap < 9; ++tap) {
                const float wr = __bfloat162float(__float2bfloat16_rn(w[(tap * kC + oc) * 2]));
                const float wi = __bfloat162float(__float2bfloat16_rn(w[(tap * kC + oc) * 2 + 1]));
                ar += wr * xr[tap] - wi * xi[tap];
                ai += wi * xr[tap] + wr * xi[tap];
            }
            o[oc] = __float2bfloat16_rn(fmaxf(ar, 0.0f));
            o[kC + oc] = __float2bfloat16_rn(fmaxf(ai, 0.0f));
        }
    }
}

// Last layer: d = conv(h5; C -> 1) + b; psi_out = psi + s d (FP32).  With a
// target, writes the loss terms and g = dL/dd (FP32 [B][H][W][2]).
__global__ void last_layer_kernel(const __nv_bfloat16 *__restrict__ h, const float *__restrict__ wl,
                                  const float2 *__restrict__ psi, const float *__restrict__ s_img,
                                  const float2 *__restrict__ target, float2 *__restrict__ out, float *__restrict__ g,
                                  double *__restrict__ loss_part, float gscale, int B, int H, int W) {
    __shared__ float w[9 * kC * 2 + 2];
    __shared__ double red[256];
    for (int i = threadIdx.x; i < 9 * kC * 2 + 2; i += blockDim.x) {
        const float v = wl[i];
        w[i] = i < 9 * kC * 2 ? __bfloat162float(__float2bfloat16_rn(v)) : v;
    }
    __syncthreads();
    const size_t npix = (size_t)B * H * W;
    double acc = 0.0;
    for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < npix; p += (size_t)gridDim.x * blockDim.x) {
        const int b = (int)(p / ((size_t)H * W)), y = (int)((p / W) % H), x = (int)(p % W);
        float dr = w[9 * kC * 2], di = w[9 * kC * 2 + 1];
        for (int tap = 0; tap < 9; ++tap) {
            const int yy = (y + tap / 3 - 1 + H) % H, xx = (x + tap % 3 - 1 + W) % W;
            const __nv_bfloat16 *hp = h + (((size_t)b * H + yy) * W + xx) * 64;
            const float *wt = w + tap * kC * 2;
#pragma unroll 8
            for (int ic = 0; ic < kC; ++ic) {
                const float hr = bf(hp[ic]), hi = bf(hp[kC + ic]);
                dr += wt[ic * 2] * hr - wt[ic * 2 + 1] * hi;
                di += wt[ic * 2 + 1] * hr + wt[ic * 2] * hi;
            }
        }
        const float s = s_img[b];
        if (out) {
            const float2 v = psi[p];
            out[p] = make_float2(v.x + s * dr, v.y + s * di);
        }
        if (target) {
            // target residual in the network's units: (fine - coarse) / s
            const float2 f = target[p], c = psi[p];
            const float er = dr - (f.x - c.x) / s, ei = di - (f.y - c.y) / s;
            acc += (double)er * er + (double)ei * ei;
            g[p * 2] = gscale * er;
            g[p * 2 + 1] = gscale * ei;
        }
    }
    if (loss_part) {
        red[threadIdx.x] = acc;
        __syncthreads();
        for (int k = blockDim.x / 2; k > 0; k >>= 1) {
            if ((int)threadIdx.x < k) red[threadIdx.x] += red[threadIdx.x + k];
            __syncthreads();
        }
        if (threadIdx.x == 0) loss_part[blockIdx.x] = red[0];
    }
}

// Input gradient of the last layer, masked by h5 > 0: dh5 = mask * conv^T(g).
__global__ void last_layer_dx_kernel(const float *__restrict__ g, const float *__restrict__ wl,
                                     const __nv_bfloat16 *__restrict__ h5, __nv_bfloat16 *__restrict__ dh,
                                     int B, int H, int W) {
    __shared__ float w[9 * kC * 2];
    for (int i = threadIdx.x; i < 9 * kC * 2; i += blockDim.x) w[i] = __bfloat162float(__float2bfloat16_rn(wl[i]));
    __syncthreads();
    const size_t npix = (size_t)B * H * W;
    for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < npix; p += (size_t)gridDim.x * blockDim.x) {
        const int b = (int)(p / ((size_t)H * W)), y = (int)((p / W) % H), x = (int)(p % W);
        float gr[9], gi[9];
#pragma unroll
        for (int tap = 0; tap < 9; ++tap) {
            // output pixel q = p - tap offset sees this pixel through tap
            const int yy = (y - (tap / 3 - 1) + H) % H, xx = (x - (tap % 3 - 1) + W) % W;
            const size_t q = ((size_t)b * H + yy) * W + xx;
            gr[tap] = g[q * 2];
            gi[tap] = g[q * 2 + 1];
        }
        const __nv_bfloat16 *m = h5 + p * 64;
        __nv_bfloat16 *o = dh + p * 64;
        for (int ic = 0; ic < kC; ++ic) {
            float ar = 0.f, ai = 0.f;
#pragma unroll
            for (int tap = 0; tap < 9; ++tap) {
                const float wr = w[(tap * kC + ic) * 2], wi = w[(tap * kC + ic) * 2 + 1];
                // d = sum W h: dL/dhr = wr gr + wi gi, dL/dhi = -wi gr + wr gi
                ar += wr * gr[tap] + wi * gi[tap];
                ai += -wi * gr[tap] + wr * gi[tap];
            }
            o[ic] = __float2bfloat16_rn(bf(m[ic]) > 0.f ? ar : 0.f);
            o[kC + ic] = __float2bfloat16_rn(bf(m[kC + ic]) > 0.f ? ai : 0.f);
        }
    }
}

// Weight gradient partial sums: dW[tap][n][k] = sum_p dy[p][n] x[p + tap][k]
// over pixel block `blockIdx.y`; nr, kr real channel counts (<= 64); dy and x
// bf16 ([p][ldy], [p][ldx]) or, for the last layer, dy as FP32 (dyf).  Bias
// gradient (sum_p dy[p][n]) in row 9 of the partial.  Each CTA handles one
// tap (blockIdx.x = tap) and writes partial[block][tap][n][k].
constexpr int kDwPix = 64;    // pixels staged per step
constexpr int kDwBlockPix = 16384;  // pixels per partial-sum block
__global__ void dw_kernel(const __nv_bfloat16 *__restrict__ dy, const float *__restrict__ dyf, int ldy,
                          const __nv_bfloat16 *__restrict__ x, int ldx, int nr, int kr, int B, int H, int W,
                          int pix_per_block, float *__restrict__ partial) {
    __shared__ float sdy[kDwPix][65];
    __shared__ float sx[kDwPix][65];
    const int tap = blockIdx.x;  // 0..8, 9 = bias
    const size_t npix = (size_t)B * H * W;
    const size_t p0 = (size_t)blockIdx.y * pix_per_block;
    const size_t p1 = p0 + pix_per_block < npix ? p0 + pix_per_block : npix;
    // each thread owns up to 4 x 4 (n, k) entries
    const int tn = threadIdx.x / 16, tk = threadIdx.x % 16;
    float acc[4][4] = {};
    for (size_t pb = p0; pb < p1; pb += kDwPix) {
        const int cnt = (int)(p1 - pb < (size_t)kDwPix ? p1 - pb : (size_t)kDwPix);
        {
            const int c = threadIdx.x % 64;
            for (int r = threadIdx.x / 64; r < kDwPix; r += blockDim.x / 64) {
                float vy = 0.f, vx = 0.f;
                if (r < cnt) {
                    const size_t p = pb + r;
                    if (c < nr) vy = dyf ? dyf[p * ldy + c] : bf(dy[p * ldy + c]);
                    if (c < kr) {
                        if (tap < 9) {
                            const int b = (int)(p / ((size_t)H * W)), y = (int)((p / W) % H), xq = (int)(p % W);
                            const int yy = (y + tap / 3 - 1 + H) % H, xx = (xq + tap % 3 - 1 + W) % W;
                            vx = bf(x[(((size_t)b * H + yy) * W + xx) * ldx + c]);
                        } else {
                            vx = 1.0f;
                        }
                    }
                }
                sdy[r][c] = vy;
                sx[r][c] = vx;
            }
        }
        __syncthreads();
        for (int r = 0; r < cnt; ++r) {
            float a[4], bq[4];
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                a[j] = sdy[r][tn * 4 + j];
                bq[j] = sx[r][tk * 4 + j];
            }
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) acc[i][j] += a[i] * bq[j];
        }
        __syncthreads();
    }
    float *out = partial + ((size_t)blockIdx.y * 10 + tap) * 64 * 64;
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) out[(tn * 4 + i) * 64 + tk * 4 + j] = acc[i][j];
}

// Sum partials in block order: dw[tap][n][k] (n < nr, k < kr), bias grad from row 9 (k = 0).
__global__ void dw_reduce_kernel(const float *__restrict__ partial, int nblocks, int nr, int kr,
                                 float *__restrict__ dw, float *__restrict__ db) {
    const int total = 9 * nr * kr + nr;
    for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < total; idx += gridDim.x * blockDim.x) {
        int tap, n, k;
        if (idx < 9 * nr * kr) {
            tap = idx / (nr * kr);
            n = (idx / kr) % nr;
            k = idx % kr;
        } else {
            tap = 9;
            n = idx - 9 * nr * kr;
            k = 0;
        }
        double s = 0.0;
        for (int b = 0; b < nblocks; ++b) s += partial[(((size_t)b * 10 + tap) * 64 + n) * 64 + k];
        if (tap < 9) dw[idx] = (float)s;
        else db[n] = (float)s;
    }
}

// bias gradient (complex): db_c[o] = (db[o], db[co + o])
__global__ void bias_contract_kernel(const float *db, int co, float *g) {
    const int o = blockIdx.x * blockDim.x + threadIdx.x;
    if (o < co) {
        g[o * 2] = db[o];
        g[o * 2 + 1] = db[co + o];
    }
}

// first layer's weight gradient needs dy = dh1 (bf16 [p][64]) and x = xin ([p][2])
// -> handled by dw_kernel with kr = 2.

// Per-image scale s = sqrt(sum |psi|^2 / 256^2) (and 1/s): the wave's norm over
// a fixed reference area of 256^2 pixels, so a probe keeps its per-pixel scale
// whatever the grid it is computed on.
constexpr double kRefPixels = 65536.0;
__global__ void rms_kernel(const float2 *__restrict__ psi, int HW, float *__restrict__ s, float *__restrict__ inv) {
    __shared__ double red[256];
    const int b = blockIdx.x;
    double acc = 0.0;
    for (int i = threadIdx.x; i < HW; i += blockDim.x) {
        const float2 v = psi[(size_t)b * HW + i];
        acc += (double)v.x * v.x + (double)v.y * v.y;
    }
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int k = blockDim.x / 2; k > 0; k >>= 1) {
        if ((int)threadIdx.x < k) red[threadIdx.x] += red[threadIdx.x + k];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        double r = sqrt(red[0] / kRefPixels);
        if (!(r > 0)) r = 1.0;
        s[b] = (float)r;
        inv[b] = (float)(1.0 / r);
    }
}

__global__ void adam_kernel(float *__restrict__ p, const float *__restrict__ g, float *__restrict__ m,
                            float *__restrict__ v, int n, float lr, float b1, float b2, float eps, float c1, float c2) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float gi = g[i];
        const float mi = b1 * m[i] + (1.f - b1) * gi;
        const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    }
}

}  // namespace closure

// ------------------------------------------------------------------ host side
using namespace closure;

namespace {
inline int grid_for(size_t n, int threads, int nsm) {
    size_t g = (n + threads - 1) / threads;
    const size_t cap = (size_t)nsm * 8;
    return (int)(g < cap ? (g > 0 ? g : 1) : cap);
}
}  // namespace

int closure_param_count() { return param_count(); }

cudaError_t ClosureNet::alloc_params() {
    const size_t n = (size_t)param_count();
    cudaError_t e;
    if ((e = cudaMalloc(&params, sizeof(float) * n)) != cudaSuccess) return e;
    if ((e = cudaMalloc(&grads, sizeof(float) * n)) != cudaSuccess) return e;
    if ((e = cudaMalloc(&adam_m, sizeof(float) * n)) != cudaSuccess) return e;
    if ((e = cudaMalloc(&adam_v, sizeof(float) * n)) != cudaSuccess) return e;
    if ((e = cudaMemset(adam_m, 0, sizeof(float) * n)) != cudaSuccess) return e;
    if ((e = cudaMemset(adam_v, 0, sizeof(float) * n)) != cudaSuccess) return e;
    // expanded bf16 weights of the four tensor-core layers, forward and transposed
    if ((e = cudaMalloc(&wt, sizeof(__nv_bfloat16) * 8 * 9 * 64 * 64)) != cudaSuccess) return e;
    if ((e = cudaMalloc(&dwreal, sizeof(float) * (9 * 64 * 64 + 64))) != cudaSuccess) return e;
    return cudaSuccess;
}

void ClosureNet::release() {
    void *ptrs[] = {params, grads, adam_m, adam_v, wt, dwreal, acts, partial, loss_part, scale};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    params = grads = adam_m = adam_v = dwreal = partial = scale = nullptr;
    wt = nullptr;
    acts = nullptr;
    loss_part = nullptr;
    cap_pix = 0;
    cap_img = 0;
}

// Workspace for `npix` pixels of `nimg` images: training keeps every layer's
// activation; inference only a ping-pong pair.
cudaError_t ClosureNet::ensure(size_t npix, int nimg, bool train) {
    const size_t per_pix = train ? (2 * 2 + 5 * 128 + 2 * 128 + 8) : (2 * 128);
    if (npix > cap_pix || (train && !cap_train) || nimg > cap_img) {
        if (acts) cudaFree(acts);
        if (partial) cudaFree(partial);
        if (loss_part) cudaFree(loss_part);
        if (scale) cudaFree(scale);
        acts = nullptr;
        partial = nullptr;
        loss_part = nullptr;
        scale = nullptr;
        cap_pix = 0;
        cap_img = 0;
        cudaError_t e;
        if ((e = cudaMalloc(&acts, per_pix * npix + 1024)) != cudaSuccess) return e;
        const size_t nblk = (npix + kDwBlockPix - 1) / kDwBlockPix;
        if ((e = cudaMalloc(&partial, sizeof(float) * nblk * 10 * 64 * 64)) != cudaSuccess) return e;
        if ((e = cudaMalloc(&loss_part, sizeof(double) * 4096)) != cudaSuccess) return e;
        if ((e = cudaMalloc(&scale, sizeof(float) * 2 * nimg)) != cudaSuccess) return e;
        cap_pix = npix;
        cap_img = nimg;
        cap_train = train;
    }
    return cudaSuccess;
}

cudaError_t ClosureNet::expand(cudaStream_t s, int nsm, int64_t *launches) {
    // layers 1..4 (0-based) are the tensor-core layers; slot 2j forward, 2j+1 transposed
    for (int l = 1; l <= 4; ++l) {
        const float *wl = params + param_offset(l);
        __nv_bfloat16 *f = wt + (size_t)(2 * (l - 1)) * 9 * 64 * 64;
        expand_kernel<<<grid_for(9 * 64 * 64, 256, nsm), 256, 0, s>>>(wl, kC, kC, 0, f);
        expand_kernel<<<grid_for(9 * 64 * 64, 256, nsm), 256, 0, s>>>(wl, kC, kC, 1, f + 9 * 64 * 64);
        *launches += 2;
    }
    return cudaGetLastError();
}

cudaError_t ClosureNet::conv_tc(const __nv_bfloat16 *in, const __nv_bfloat16 *w, const float *bias,
                                const __nv_bfloat16 *mask, __nv_bfloat16 *out, int B, int H, int W, int epi,
                                int *err, cudaStream_t s, int nsm, int64_t *launches) {
    static KernelSetup ks;
    int per_sm = 0;
    cudaError_t e = ks.get(conv_tc_kernel, 128, kConvSmem, true, &per_sm);
    if (e != cudaSuccess) return e;
    // two CTAs fit an SM by shared memory (105 KB each) and registers; the
    // occupancy query answers one for this tensor-memory kernel, so the grid
    // asks for two (a CTA that does not fit waits for a free slot)
    static_assert(2 * (kConvSmem + 2048) <= 233472, "two conv CTAs fit an SM");
    if (per_sm < 2) per_sm = 2;
    const int ntiles = B * H * (W / kTile);
    int grid = nsm * per_sm < ntiles ? nsm * per_sm : ntiles;
    ++*launches;
    conv_tc_kernel<<<grid, 128, kConvSmem, s>>>(in, w, bias, mask, out, B, H, W, epi, err);
    return cudaGetLastError();
}

// Forward pass.  psi: complex64 [B][H][W]; out (may be null, may equal psi):
// psi + s d; target (training): the fine-slice waves -> loss and dL/dd.
cudaError_t ClosureNet::forward(const float2 *psi, int B, int H, int W, float2 *out, const float2 *target,
                                bool train, int *err, cudaStream_t s, int nsm, int64_t *launches) {
    if (W % kTile || H < 3 || W < 3) return cudaErrorInvalidValue;
    const size_t npix = (size_t)B * H * W;
    cudaError_t e = ensure(npix, B, train);
    if (e != cudaSuccess) return e;
    if ((e = expand(s, nsm, launches)) != cudaSuccess) return e;
    float *sc = scale, *inv = scale + B;
    rms_kernel<<<B, 256, 0, s>>>(psi, H * W, sc, inv);
    ++*launches;
    __nv_bfloat16 *h[6];
    __nv_bfloat16 *x0;
    unsigned char *a = (unsigned char *)acts;
    if (train) {
        x0 = (__nv_bfloat16 *)a;
        a += ((npix * 4 + 255) / 256) * 256;
        for (int l = 1; l <= 5; ++l) {
            h[l] = (__nv_bfloat16 *)a;
            a += npix * 128;
        }
        dh[0] = (__nv_bfloat16 *)a;
        a += npix * 128;
        dh[1] = (__nv_bfloat16 *)a;
        a += npix * 128;
        g6 = (float *)a;
    } else {
        // inference: h1 -> A, h2 -> B, h3 -> A, ... ; the scaled input is not kept
        x0 = nullptr;
        h[1] = h[3] = h[5] = (__nv_bfloat16 *)a;
        h[2] = h[4] = (__nv_bfloat16 *)(a + npix * 128);
        g6 = nullptr;
    }
    for (int l = 1; l <= 5; ++l) hbuf[l] = h[l];
    xbuf = x0;
    __nv_bfloat16 *xin_scratch = x0;
    if (!train) {
        // first_layer_kernel writes the scaled bf16 input too: give it the B buffer's tail
        // region (h2 is written only after h1 is complete)
        xin_scratch = h[2];
    }
    first_layer_kernel<<<grid_for(npix, 256, nsm), 256, 0, s>>>(psi, inv, params + param_offset(0), xin_scratch,
                                                                   h[1], B, H, W);
    ++*launches;
    for (int l = 1; l <= 4; ++l) {
        const __nv_bfloat16 *w = wt + (size_t)(2 * (l - 1)) * 9 * 64 * 64;
        const float *bias = params + param_offset(l) + layer_wsize(l);
        if ((e = conv_tc(h[l], w, bias, nullptr, h[l + 1], B, H, W, EPI_BIAS_RELU, err, s, nsm, launches)) !=
            cudaSuccess)
            return e;
    }
    const int nblk = grid_for(npix, 256, nsm);
    last_layer_kernel<<<nblk, 256, 0, s>>>(h[5], params + param_offset(5), psi, sc, target, out,
                                           target ? g6 : nullptr, target ? loss_part : nullptr,
                                           target ? 2.0f / (float)npix : 0.f, B, H, W);
    ++*launches;
    loss_blocks = target ? nblk : 0;
    return cudaGetLastError();
}

// Backward pass after forward(train = true, target): grads <- dL/dtheta.
cudaError_t ClosureNet::backward(int B, int H, int W, int *err, cudaStream_t s, int nsm, int64_t *launches) {
    const size_t npix = (size_t)B * H * W;
    const int nblk = (int)((npix + kDwBlockPix - 1) / kDwBlockPix);
    cudaError_t e;
    auto wgrad = [&](int l, const __nv_bfloat16 *dy, const float *dyf, int ldy, const __nv_bfloat16 *x, int ldx) {
        const int co = layer_co(l), ci = layer_ci(l);
        dw_kernel<<<dim3(10, nblk), 256, 0, s>>>(dy, dyf, ldy, x, ldx, 2 * co, 2 * ci, B, H, W, kDwBlockPix,
                                                 partial);
        dw_reduce_kernel<<<grid_for(9 * 4 * co * ci + 2 * co, 256, nsm), 256, 0, s>>>(
            partial, nblk, 2 * co, 2 * ci, dwreal, dwreal + 9 * 64 * 64);
        float *g = grads + param_offset(l);
        contract_kernel<<<grid_for(9 * co * ci, 256, nsm), 256, 0, s>>>(dwreal, co, ci, g);
        bias_contract_kernel<<<1, 64, 0, s>>>(dwreal + 9 * 64 * 64, co, g + layer_wsize(l));
        *launches += 4;
    };
    // layer 6 (C -> 1): dW from g6, then dh5 = mask(h5) conv6^T(g6)
    wgrad(5, nullptr, g6, 2, hbuf[5], 64);
    last_layer_dx_kernel<<<grid_for(npix, 256, nsm), 256, 0, s>>>(g6, params + param_offset(5), hbuf[5], dh[1], B, H,
                                                                  W);
    ++*launches;
    int cur = 1;
    for (int l = 4; l >= 1; --l) {
        // dh[cur] = dL/dpre_{l+1} (masked); weight gradient of layer l with input h_l
        wgrad(l, dh[cur], nullptr, 64, hbuf[l], 64);
        const __nv_bfloat16 *wT = wt + (size_t)(2 * (l - 1) + 1) * 9 * 64 * 64;
        if ((e = conv_tc(dh[cur], wT, nullptr, hbuf[l], dh[cur ^ 1], B, H, W, EPI_MASK, err, s, nsm, launches)) !=
            cudaSuccess)
            return e;
        cur ^= 1;
    }
    // layer 1 (1 -> C): input the scaled bf16 wave
    wgrad(0, dh[cur], nullptr, 64, xbuf, 2);
    return cudaGetLastError();
}

cudaError_t ClosureNet::adam(float lr, cudaStream_t s, int nsm, int64_t *launches) {
    ++step;
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = 1.f - powf(b1, (float)step), c2 = 1.f - powf(b2, (float)step);
    const int n = param_count();
    adam_kernel<<<grid_for(n, 256, nsm), 256, 0, s>>>(params, grads, adam_m, adam_v, n, lr, b1, b2, 1e-8f, c1, c2);
    ++*launches;
    return cudaGetLastError();
}

// He-style initial weights from the library's splitmix64 stream (host), zero biases.
void closure_init_params(uint64_t seed, std::vector<float> &h) {
    h.assign(param_count(), 0.f);
    auto mix = [](uint64_t x) {
        x += 0x9E3779B97F4A7C15ull;
        x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
        x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
        return x ^ (x >> 31);
    };
    uint64_t ctr = 0;
    for (int l = 0; l < kLayers; ++l) {
        const int co = layer_co(l), ci = layer_ci(l);
        // complex fan-in 9 ci; the last layer starts small so the closure starts near identity
        float sd = sqrtf(1.0f / (9.0f * ci));
        if (l == kLayers - 1) sd *= 0.1f;
        float *w = h.data() + param_offset(l);
        for (int i = 0; i < 9 * co * ci * 2; ++i) {
            const double u1 = ((mix(seed ^ mix(ctr++)) >> 11) + 1.0) * (1.0 / 9007199254740993.0);
            const double u2 = (mix(seed ^ mix(ctr++)) >> 11) * (1.0 / 9007199254740992.0);
            w[i] = (float)(sd * sqrt(-2.0 * log(u1)) * cos(2.0 * 3.14159265358979323846 * u2));
        }
    }
}

}  // namespace msl
