// STEM slice loop with each probe's wave resident on chip across all slices.
//
// The streaming passes (msl_passes.cu) read and write every probe's wave from
// HBM twice per slice (32 N^2 bytes per probe-slice).  Here one thread-block
// cluster of 8 CTAs owns one probe at a time: a 256 x 256 complex64 wave
// (512 KB) is split by rows (ix) over the 8 CTAs' shared memory, 32 lines
// (64 KB) each, and stays there from the first slice to the detector.  Per
// slice (mulslice.cpp:706-739):
//   A  each CTA transforms its own 32 lines along iy: ifft_y, * t, fft_y (the
//      streaming row pass's half-warp, radix 16 x 16 transform);
//   push: its rows, stored as 8 blocks of 32 rows x 32 columns (8 KB, block q
//      holding the columns CTA q owns), go to the CTAs that own those columns
//      by 8 bulk copies through distributed shared memory
//      (cp.async.bulk.shared::cluster), each completing on the receiver's
//      mbarrier;
//   B  once its 64 KB have arrived, each CTA transforms its 32 columns along
//      ix: fft_x, propagator and band limit, [detector sums], ifft_x;
//   write-back: the column blocks return to the row owners the same way.
// No cluster barrier runs inside a probe's slice loop: every block a CTA
// overwrites has provably been read (the receiver's mbarrier of the copy that
// read it completed before the copy that overwrites it was issued), so the
// wave's only HBM traffic is the probe read once and the transmission rows
// (8 N^2 bytes per slice, shared through L2 by every cluster on the same
// slice).  Blocks keep element (r, c) at slot r * 32 + (c ^ (r & 15)), which
// keeps both the row transform's and the column transform's 16-lane accesses
// on 16 distinct bank pairs; line transforms exchange through a separate 64 KB
// area.  Detector sums: FP64 per thread, per warp, per CTA, in a fixed order;
// the per-CTA partials are added by the scan's finalize kernel.
#include <cuda_runtime.h>
#include <stdint.h>

#include "msl_fft.cuh"
#include "msl_internal.h"
#include "msl_tma.cuh"

namespace msl {

namespace {

using RP = HalfWarpPlan256;
constexpr int kN = 256, kCL = 8, kLines = kN / kCL, kThreads = 16 * kLines, kMaxDetR = 8;
constexpr size_t kLineBytes = sizeof(float2) * kN;                 // 2 KB, also the exchange alignment
constexpr size_t kBlock = sizeof(float2) * kLines * kLines;         // 8 KB: 32 rows x 32 columns
constexpr size_t kOffR = 0;                                         // row blocks [dest q][r][c] (64 KB)
constexpr size_t kOffS = kOffR + kCL * kBlock;                      // column blocks [src p][r][c] (64 KB)
constexpr size_t kOffX = kOffS + kCL * kBlock;                      // 32 line exchange areas (64 KB)
constexpr size_t kOffTw = kOffX + kLines * kLineBytes;              // 16 x 16 stage-1 table
constexpr size_t kOffRed = kOffTw + sizeof(float2) * 256;           // per-warp detector sums
constexpr size_t kOffBar = kOffRed + sizeof(double) * (kThreads / 32) * kMaxDetR;
constexpr size_t kResidentSmem = kOffBar + 2 * sizeof(uint64_t) + kLineBytes;
static_assert(kResidentSmem <= 227 * 1024, "shared memory");
constexpr uint32_t kResWait = 1u << 22;

__device__ __forceinline__ uint32_t cluster_rank() {
    uint32_t r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return r;
}
__device__ __forceinline__ uint32_t cluster_id_x() {
    uint32_t r;
    asm volatile("mov.u32 %0, %%clusterid.x;" : "=r"(r));
    return r;
}
__device__ __forceinline__ uint32_t nclusters_x() {
    uint32_t r;
    asm volatile("mov.u32 %0, %%nclusterid.x;" : "=r"(r));
    return r;
}
__device__ __forceinline__ void cluster_arrive() {
    asm volatile("barrier.cluster.arrive.release.aligned;" ::: "memory");
}
__device__ __forceinline__ void cluster_wait() {
    asm volatile("barrier.cluster.wait.acquire.aligned;" ::: "memory");
}
__device__ __forceinline__ uint32_t map_rank(uint32_t addr, uint32_t rank) {
    uint32_t r;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(addr), "r"(rank));
    return r;
}
// slot of element (r, c) inside a block
__device__ __forceinline__ uint32_t bslot(int r, int c) { return (uint32_t)(r * kLines + (c ^ (r & 15))); }
// bulk copy from this CTA's shared memory to a cluster peer's, completing on the peer's mbarrier
__device__ __forceinline__ void bulk_to_peer(uint32_t dst_cluster, uint32_t src, uint32_t bytes, uint32_t bar_cluster) {
    asm volatile(
        "cp.async.bulk.shared::cluster.shared::cta.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            dst_cluster),
        "r"(src), "r"(bytes), "r"(bar_cluster)
        : "memory");
}
}  // namespace

__global__ void __launch_bounds__(kThreads, 1) stem_resident_kernel(ResidentArgs a) {
    extern __shared__ unsigned char smraw[];
    const uint32_t AL = (uint32_t)kLineBytes;
    unsigned char *base = smraw + ((AL - (smem_u32(smraw) & (AL - 1u))) & (AL - 1u));
    float2 *R = reinterpret_cast<float2 *>(base + kOffR);
    float2 *S = reinterpret_cast<float2 *>(base + kOffS);
    float2 *tw = reinterpret_cast<float2 *>(base + kOffTw);
    double *red = reinterpret_cast<double *>(base + kOffRed);
    uint64_t *barS = reinterpret_cast<uint64_t *>(base + kOffBar), *barR = barS + 1;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, t = lane & 15;
    const int j = 2 * warp + (lane >> 4);  // this half-warp's row line / column (0..31)
    const uint32_t rank = cluster_rank();
    for (int i = tid; i < 256; i += kThreads) {
        float sn, cn;
        sincospif((float)(2 * (i / 16) * (i % 16)) / (float)kN, &sn, &cn);  // exp(2 pi i r k / N), [r][k]
        tw[i] = make_float2(cn, sn);
    }
    if (tid == 0) {
        mbar_init(barS, 1);
        mbar_init(barR, 1);
        mbar_fence_init();
    }
    __syncthreads();
    cluster_arrive();  // every CTA's mbarriers exist before any peer copies toward them
    cluster_wait();
    const uint32_t Rs = smem_u32(R), Ss = smem_u32(S);
    const int ix_row = (int)rank * kLines + j;   // phase A: this half-warp's line
    const int iy_col = (int)rank * kLines + j;   // phase B: this half-warp's column
    const RowXorLin<RP> adX{smem_u32(base + kOffX) + (uint32_t)(j * kLineBytes)};
    const float ky2 = a.ky2[iy_col];
    uint32_t ps = 0, pr = 0;
    bool ok = true;
    for (int b = (int)cluster_id_x(); b < a.nprobe; b += (int)nclusters_x()) {
        int ic = 0;
        for (int s = 0; s < a.nslice; ++s) {
            const int l = a.layer_seq[s];
            // ---- A: the row line ix_row (element iy = t + 16 e: block e >> 1, column t + 16 (e & 1))
            float2 v[RP::E];
            if (s == 0) {
                const float2 *src = a.w0 + ((size_t)b * kN + ix_row) * kN;
#pragma unroll
                for (int e = 0; e < RP::E; ++e) v[e] = src[t + 16 * e];
            } else {
                if (!mbar_wait_bounded(barR, pr, kResWait)) ok = false;
                pr ^= 1u;
#pragma unroll
                for (int e = 0; e < RP::E; ++e) v[e] = R[(e >> 1) * kLines * kLines + bslot(j, t + 16 * (e & 1))];
            }
            // the transmission row is requested before the inverse transform, so its
            // L2 latency hides behind it
            const float2 *trow = a.trans + ((size_t)l * kN + ix_row) * kN;
            float2 tv[RP::E];
#pragma unroll
            for (int e = 0; e < RP::E; ++e) tv[e] = __ldg(trow + t + 16 * e);
            fft_line_tab<RP, -1>(v, t, adX, tw);
#pragma unroll
            for (int e = 0; e < RP::E; ++e) v[e] = c_mul(v[e], tv[e]);
            fft_line_tab<RP, +1>(v, t, adX, tw);
#pragma unroll
            for (int e = 0; e < RP::E; ++e) R[(e >> 1) * kLines * kLines + bslot(j, t + 16 * (e & 1))] = v[e];
            fence_proxy_async();
            __syncthreads();
            if (tid == 0) {
                mbar_arrive_expect_tx(barS, (uint32_t)(kCL * kBlock));
                for (int q = 0; q < kCL; ++q)
                    bulk_to_peer(map_rank(Ss + (uint32_t)(rank * kBlock), (uint32_t)q), Rs + (uint32_t)(q * kBlock),
                                 (uint32_t)kBlock, map_rank(smem_u32(barS), (uint32_t)q));
            }
            // ---- B: the column iy_col (element ix = t + 16 e: block e >> 1, row t + 16 (e & 1))
            if (!mbar_wait_bounded(barS, ps, kResWait)) ok = false;
            ps ^= 1u;
#pragma unroll
            for (int e = 0; e < RP::E; ++e) v[e] = S[(e >> 1) * kLines * kLines + bslot(t + 16 * (e & 1), j)];
            // propagator factors requested before the forward transform (their latency hides behind it)
            const float2 *px = a.prop + (size_t)l * 2 * kN, *py = px + kN;
            const float2 pyv = __ldg(py + iy_col);
            float2 pv[RP::E];
#pragma unroll
            for (int e = 0; e < RP::E; ++e) pv[e] = __ldg(px + t + 16 * e);
            fft_line_tab<RP, +1>(v, t, adX, tw);
#pragma unroll
            for (int e = 0; e < RP::E; ++e) {
                const int ix = t + 16 * e;
                const float k2 = a.kx2[ix] + ky2;
                v[e] = k2 < a.k2max ? c_mul(c_mul(v[e], pyv), pv[e]) : make_float2(0.f, 0.f);
            }
            const bool detect = ic < a.ncheck && a.checkpoints[ic] == s;
            if (detect) {
                double acc[kMaxDetR];
#pragma unroll
                for (int d = 0; d < kMaxDetR; ++d) acc[d] = 0.0;
#pragma unroll
                for (int e = 0; e < RP::E; ++e) {
                    const int ix = t + 16 * e;
                    const uint32_t m = a.mask[(size_t)ix * kN + iy_col];
                    const double p = (double)v[e].x * v[e].x + (double)v[e].y * v[e].y;
#pragma unroll
                    for (int d = 0; d < kMaxDetR; ++d)
                        if (m & (1u << d)) acc[d] += p;
                }
#pragma unroll
                for (int d = 0; d < kMaxDetR; ++d) {
                    double x = acc[d];
#pragma unroll
                    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
                    if (lane == 0) red[warp * kMaxDetR + d] = x;
                }
                __syncthreads();
                if (tid < a.ndet) {
                    double x = 0.0;
                    for (int w = 0; w < kThreads / 32; ++w) x += red[w * kMaxDetR + tid];
                    a.partial[(((size_t)ic * a.nprobe + b) * kCL + rank) * a.ndet + tid] = x;
                }
                ++ic;
            }
            const bool last = s == a.nslice - 1 || ic >= a.ncheck;
            if (last) break;
            fft_line_tab<RP, -1>(v, t, adX, tw);
            // ---- write-back: the column blocks to their row owners
#pragma unroll
            for (int e = 0; e < RP::E; ++e) S[(e >> 1) * kLines * kLines + bslot(t + 16 * (e & 1), j)] = v[e];
            fence_proxy_async();
            __syncthreads();
            if (tid == 0) {
                mbar_arrive_expect_tx(barR, (uint32_t)(kCL * kBlock));
                for (int p = 0; p < kCL; ++p)
                    bulk_to_peer(map_rank(Rs + (uint32_t)(rank * kBlock), (uint32_t)p), Ss + (uint32_t)(p * kBlock),
                                 (uint32_t)kBlock, map_rank(smem_u32(barR), (uint32_t)p));
            }
        }
        // the probe's last column blocks are read, every copy of this probe has landed:
        // the next probe may overwrite rows and columns everywhere in the cluster
        __syncthreads();
        cluster_arrive();
        cluster_wait();
    }
    if (!ok && a.err) atomicExch(a.err, 1);
}

cudaError_t launch_stem_resident(const ResidentArgs &a, cudaStream_t s, int nsm, int64_t *launches) {
    static KernelSetup ks;
    int per_sm = 0;
    cudaError_t e = ks.get(stem_resident_kernel, kThreads, kResidentSmem, true, &per_sm);
    if (e != cudaSuccess) return e;
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = kCL;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.blockDim = dim3(kThreads, 1, 1);
    cfg.dynamicSmemBytes = kResidentSmem;
    cfg.stream = s;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    int nclusters = 0;
    cfg.gridDim = dim3(kCL, 1, 1);
    e = cudaOccupancyMaxActiveClusters(&nclusters, stem_resident_kernel, &cfg);
    if (e != cudaSuccess) return e;
    if (nclusters < 1) return cudaErrorInvalidConfiguration;
    if (nclusters > a.nprobe) nclusters = a.nprobe;
    cfg.gridDim = dim3(kCL * nclusters, 1, 1);
    ++*launches;
    e = cudaLaunchKernelEx(&cfg, stem_resident_kernel, a);
    if (e != cudaSuccess) return e;
    return cudaGetLastError();
}

int resident_side() { return kN; }
int resident_cluster() { return kCL; }

}  // namespace msl
