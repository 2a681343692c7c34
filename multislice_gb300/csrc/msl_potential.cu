// Projected-potential gather kernel: the PotentialBuilder step.
//
// Reference: LMultiSlice ModelPotential::calculatePotentialGrid
// (ImageSimulation/LMultiSlice/ModelPotential.cu:27-99) bins atoms by z and, for
// every pixel, sums calculateProjectedPotential over all atoms of the slice in
// 4608-atom constant-memory batches (:125-230), evaluating K0 in FP64 for every
// pixel-atom pair before the cutoff test.  The atom form used here is Kirkland's
// vzatom (multislice/slicelib.cpp:2666-2716):
//     V(r) = AL sum_i a_i K0(2 pi r sqrt(b_i)) + AG sum_i (c_i/d_i) exp(-pi^2 r^2 / d_i)
// with FPARAMS coefficients, K0/I0 by the Abramowitz & Stegun 9.8.1/9.8.5/9.8.6
// polynomials the reference uses (slicelib.cpp:168-235).
//
// GB300 design: one CTA per 64 x 32 pixel tile of one slice, eight pixels per
// thread (independent accumulators for latency hiding).  The slice's atoms
// stream through in rounds of 512, two per thread; each round is culled against
// the tile's periodic bounding box (in float, from float copies of the
// coordinates, with a margin that keeps every atom the exact test would:
// culling only has to be conservative) and compacted in atom order (so the
// float sum order is fixed) into a list of at most 64 atoms at a time.  Each
// atom arrives as its nearest pixel (ic, jc) and the residue x - ic dxp,
// y - jc dyp, formed on the host in FP64 and rounded to float, so the offset of
// pixel column ix is |residue + m dxp| with m = ic - ix folded to the minimum
// image in integers: all in FP32, and an atom sitting exactly on a pixel keeps
// the FP64 residue there (r is then clamped to 1e-10 A as the reference does,
// never a float rounding residue).  The per-atom offsets of the tile's 32
// columns and 32 rows are formed once per tile and the pair loop runs in FP32
// on them.  Every pixel sums its atoms in atom order, whatever the tile shape.
// 64-pixel-wide tiles halve the per-pixel share of the per-atom work against
// 32 x 32 (Au 2048^2: 2.78 ms per configuration against 3.40).
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "msl_internal.h"

namespace msl {

namespace {
// tile shape and list capacity picked by timing 16 / 32 / 64 / 128-pixel-wide tiles
// and 32 / 64 / 128-atom lists on the Au 2048^2 potentials
constexpr int TX = 64, TY = 32, THREADS = 256, PX = TX * TY / THREADS, CAP = 64;
constexpr int KR = 2, ROUND = KR * THREADS, NW = THREADS / 32;  // atoms culled per thread per round

__device__ __forceinline__ float poly(const float *c, int n, float t) {
    float s = c[n - 1];
    for (int i = n - 2; i >= 0; --i) s = fmaf(s, t, c[i]);
    return s;
}

__constant__ float kI0A[7] = {1.0f, 3.5156229f, 3.0899424f, 1.2067492f, 0.2659732f, 0.0360768f, 0.0045813f};
__constant__ float kK0A[7] = {-0.57721566f, 0.42278420f, 0.23069756f, 0.03488590f, 0.00262698f,
                              0.00010750f, 0.00000740f};
__constant__ float kK0B[7] = {1.25331414f, -0.07832358f, 0.02189568f, -0.01062446f, 0.00587872f,
                              -0.00251540f, 0.00053208f};

// K0(x), x > 0 (A&S 9.8.5 for x <= 2 with I0 from 9.8.1, 9.8.6 above).
__device__ __forceinline__ float bessk0f(float x) {
    if (x <= 2.0f) {
        const float t = (x / 3.75f) * (x / 3.75f);
        const float i0 = poly(kI0A, 7, t);
        const float x2 = 0.25f * x * x;
        return -logf(0.5f * x) * i0 + poly(kK0A, 7, x2);
    }
    return expf(-x) * poly(kK0B, 7, 2.0f / x) * rsqrtf(x);
}
}  // namespace

template <bool TAB>
__global__ void __launch_bounds__(THREADS, 4) potential_kernel(PotArgs a) {
    extern __shared__ float4 stab[];  // TAB: [nsp][kPotTabN] cubic pieces of the species' radial profiles
    __shared__ int sZ[CAP];
    __shared__ int sS[CAP];
    __shared__ int sic[CAP], sjc[CAP];
    __shared__ float sfx[CAP], sfy[CAP];
    __shared__ float sdx[CAP][TX];
    __shared__ float sdy[CAP][TY];
    __shared__ int wcount[KR * NW];
    const int tid = threadIdx.x;
    if (TAB) {
        for (int i = tid; i < a.nsp * kPotTabN; i += THREADS) stab[i] = a.tab[i];
    }
    const int ty = tid % TY, txg = tid / TY;  // pixels (txg + 8 j, ty), j < PX
    const int lane = tid & 31, warp = tid >> 5;
    const int iy0 = blockIdx.x * TY, ix0 = blockIdx.y * TX, s = blockIdx.z;

    // tile bounding box (pixel positions) for the culling, in float with a margin
    // that covers the float rounding of the coordinates (the culling only has to
    // keep every atom that can reach the tile; the pair loop tests r < radius)
    const float xc = (float)((ix0 + 0.5 * (TX - 1)) * a.dxp), hx = (float)(0.5 * (TX - 1) * a.dxp);
    const float yc = (float)((iy0 + 0.5 * (TY - 1)) * a.dyp), hy = (float)(0.5 * (TY - 1) * a.dyp);
    const float axf = (float)a.ax, byf = (float)a.by;
    const float rad = sqrtf(a.rad2) * (1.0f + 1e-5f) + 1e-3f;
    const int a0 = a.off[s], a1 = a.off[s + 1];
    float acc[PX];
#pragma unroll
    for (int j = 0; j < PX; ++j) acc[j] = 0.f;

    for (int c0 = a0; c0 < a1; c0 += ROUND) {
        // cull: atom c0 + k THREADS + tid; the kept atoms' pixel positions and
        // species are loaded right away so their latency overlaps the compaction
        bool keep[KR];
        unsigned ball[KR];
        int ia[KR], ja[KR], za[KR];
        float fxa[KR], fya[KR];
#pragma unroll
        for (int k = 0; k < KR; ++k) {
            const int ai = c0 + k * THREADS + tid;
            keep[k] = false;
            ia[k] = ja[k] = za[k] = 0;
            fxa[k] = fya[k] = 0.f;
            if (ai < a1) {
                float dx = fabsf(a.xf[ai] - xc);
                dx = fminf(dx, axf - dx);
                float dy = fabsf(a.yf[ai] - yc);
                dy = fminf(dy, byf - dy);
                keep[k] = (dx - hx < rad) && (dy - hy < rad);
                if (keep[k]) {
                    ia[k] = a.ic[ai];
                    ja[k] = a.jc[ai];
                    fxa[k] = a.fx[ai];
                    fya[k] = a.fy[ai];
                    za[k] = a.Z[ai];
                }
            }
            ball[k] = __ballot_sync(0xffffffffu, keep[k]);
        }
        __syncthreads();  // the previous round's pair loop is done with wcount and the lists
        if (lane == 0) {
#pragma unroll
            for (int k = 0; k < KR; ++k) wcount[k * NW + warp] = __popc(ball[k]);
        }
        __syncthreads();
        // order-preserving positions: atom order is (k, warp, lane)
        int pos[KR], total = 0;
#pragma unroll
        for (int k = 0; k < KR; ++k) {
            int before = 0, sum = 0;
            for (int w = 0; w < NW; ++w) {
                const int n = wcount[k * NW + w];
                if (w < warp) before += n;
                sum += n;
            }
            pos[k] = total + before + __popc(ball[k] & ((1u << lane) - 1u));
            total += sum;
        }
        for (int piece = 0; piece < total; piece += CAP) {
            if (piece > 0) __syncthreads();  // the previous piece's pair loop is done with the lists
#pragma unroll
            for (int k = 0; k < KR; ++k) {
                const int p = pos[k] - piece;
                if (keep[k] && p >= 0 && p < CAP) {
                    sZ[p] = za[k];
                    if (TAB) sS[p] = a.zslot[za[k]];
                    sic[p] = ia[k];
                    sjc[p] = ja[k];
                    sfx[p] = fxa[k];
                    sfy[p] = fya[k];
                }
            }
            __syncthreads();
            const int n = min(CAP, total - piece);
            // per-atom offsets of this tile's columns and rows: |residue + m pixel|,
            // m the pixel difference folded to the minimum image (ModelPotential.cu:154-203)
            for (int idx = tid; idx < n * TX; idx += THREADS) {
                const int k = idx / TX, i = idx % TX;
                int m = sic[k] - (ix0 + i);
                if (2 * m >= a.nx) m -= a.nx;
                else if (2 * m < -a.nx) m += a.nx;
                sdx[k][i] = fabsf(fmaf((float)m, a.dxpf, sfx[k]));
            }
            for (int idx = tid; idx < n * TY; idx += THREADS) {
                const int k = idx / TY, i = idx % TY;
                int m = sjc[k] - (iy0 + i);
                if (2 * m >= a.ny) m -= a.ny;
                else if (2 * m < -a.ny) m += a.ny;
                sdy[k][i] = fabsf(fmaf((float)m, a.dypf, sfy[k]));
            }
            __syncthreads();
            for (int k = 0; k < n; ++k) {
                // a warp holds 32 rows x 4 columns of the tile (ty = lane, the
                // columns txg + 8 j warp-uniform): an atom whose x offset puts all
                // four columns beyond the cutoff is skipped by the whole warp
                float dx[PX];
#pragma unroll
                for (int j = 0; j < PX; ++j) dx[j] = sdx[k][txg + 8 * j];
                float dxm = dx[0];
#pragma unroll
                for (int j = 1; j < PX; ++j) dxm = fminf(dxm, dx[j]);
                if (dxm * dxm >= a.rad2) continue;
                const float dy = sdy[k][ty], dy2 = dy * dy;
                if (dy2 >= a.rad2) continue;
                const float *p = a.sp + sZ[k] * 12;
                const float4 *tb = TAB ? stab + sS[k] * kPotTabN : nullptr;
#pragma unroll
                for (int j = 0; j < PX; ++j) {
                    const float r2 = fmaf(dx[j], dx[j], dy2);
                    if (r2 < a.rad2) {
                        // r = max(r, 1e-10 A) through the reciprocal square root
                        const float r2c = fmaxf(r2, 1.0e-20f);
                        const float r = r2c * rsqrtf(r2c);
                        if (TAB && r >= a.tab_r0) {
                            // cubic piece of the tabulated profile: ((c3 t + c2) t + c1) t + c0
                            const float u = fmaf(r, a.tab_inv_h, a.tab_off);
                            const int i = min((int)u, kPotTabN - 1);
                            const float t = u - (float)i;
                            const float4 c = tb[i];
                            acc[j] += fmaf(fmaf(fmaf(c.w, t, c.z), t, c.y), t, c.x);
                            continue;
                        }
                        float v = __ldg(p + 0) * bessk0f(__ldg(p + 1) * r) +
                                  __ldg(p + 2) * bessk0f(__ldg(p + 3) * r) +
                                  __ldg(p + 4) * bessk0f(__ldg(p + 5) * r);
                        const float rr = r * r;
                        v += __ldg(p + 6) * expf(-__ldg(p + 7) * rr) + __ldg(p + 8) * expf(-__ldg(p + 9) * rr) +
                             __ldg(p + 10) * expf(-__ldg(p + 11) * rr);
                        acc[j] += v;
                    }
                }
            }
        }
    }
    const int iy = iy0 + ty;
#pragma unroll
    for (int j = 0; j < PX; ++j) {
        const int ix = ix0 + txg + 8 * j;
        if (ix < a.nx && iy < a.ny) a.v[((size_t)s * a.nx + ix) * a.ny + iy] = acc[j];
    }
}

cudaError_t launch_potential(const PotArgs &a, cudaStream_t s, int64_t *launches) {
    ++*launches;
    dim3 grid((a.ny + TY - 1) / TY, (a.nx + TX - 1) / TX, a.nslice);
    if (a.nsp > 0 && a.tab) {
        const size_t smem = sizeof(float4) * (size_t)a.nsp * kPotTabN;
        static KernelSetup ks;
        int per_sm = 0;
        cudaError_t e = ks.get(potential_kernel<true>, THREADS, sizeof(float4) * kPotMaxSp * kPotTabN, true, &per_sm);
        if (e != cudaSuccess) return e;
        potential_kernel<true><<<grid, THREADS, smem, s>>>(a);
    } else {
        potential_kernel<false><<<grid, THREADS, 0, s>>>(a);
    }
    return cudaGetLastError();
}

// ------------------------------------------------------------ radial tables
namespace {
// vzatom in double (slicelib.cpp:2666-2716 with the A&S Bessel polynomials of :168-235)
double bessi0d(double x) {
    static const double c[7] = {1.0, 3.5156229, 3.0899424, 1.2067492, 0.2659732, 0.0360768, 0.0045813};
    const double t = (x / 3.75) * (x / 3.75);
    double s = c[6];
    for (int i = 5; i >= 0; --i) s = s * t + c[i];
    return s;
}
double bessk0d(double x) {
    static const double a[7] = {-0.57721566, 0.42278420, 0.23069756, 0.03488590, 0.00262698, 0.00010750, 0.00000740};
    static const double b[7] = {1.25331414, -0.07832358, 0.02189568, -0.01062446, 0.00587872, -0.00251540, 0.00053208};
    if (x <= 2.0) {
        const double t = 0.25 * x * x;
        double s = a[6];
        for (int i = 5; i >= 0; --i) s = s * t + a[i];
        return -log(0.5 * x) * bessi0d(x) + s;
    }
    const double t = 2.0 / x;
    double s = b[6];
    for (int i = 5; i >= 0; --i) s = s * t + b[i];
    return exp(-x) * s / sqrt(x);
}
double vz_double(const double *f, double r) {
    const double AL = 300.8242834, AG = 150.4121417, PIK = 3.141592654;
    const double x = 2.0 * PIK * r;
    double suml = 0.0, sumg = 0.0;
    for (int i = 0; i < 3; ++i) suml += f[2 * i] * bessk0d(x * sqrt(f[2 * i + 1]));
    const double x2 = (PIK * r) * (PIK * r);
    for (int i = 0; i < 3; ++i) sumg += f[6 + 2 * i] * exp(-x2 / f[7 + 2 * i]) / f[7 + 2 * i];
    return AL * suml + AG * sumg;
}
}  // namespace

void potential_tables(const double *fparams, const int *zlist, int nsp, double r0, double rmax, float4 *out) {
    const double h = (rmax - r0) / kPotTabN;
    for (int sidx = 0; sidx < nsp; ++sidx) {
        const double *f = fparams + zlist[sidx] * 12;
        for (int i = 0; i < kPotTabN; ++i) {
            // the cubic through the profile at t = 0, 1/3, 2/3, 1 of [r0 + i h, r0 + (i + 1) h]
            const double r = r0 + i * h;
            const double y0 = vz_double(f, r), y1 = vz_double(f, r + h / 3), y2 = vz_double(f, r + 2 * h / 3),
                         y3 = vz_double(f, r + h);
            const double c0 = y0;
            const double c1 = (-11 * y0 + 18 * y1 - 9 * y2 + 2 * y3) / 2;
            const double c2 = 9 * (2 * y0 - 5 * y1 + 4 * y2 - y3) / 2;
            const double c3 = 27 * (-y0 + 3 * y1 - 3 * y2 + y3) / 6;
            out[(size_t)sidx * kPotTabN + i] = make_float4((float)c0, (float)c1, (float)c2, (float)c3);
        }
    }
}

}  // namespace msl
