// STEM slice loop with each probe's wave resident on chip across all slices.
//
// The streaming passes (msl_passes.cu) read and write every probe's wave from
// HBM twice per slice (32 N^2 bytes per probe-slice).  Here one thread-block
// cluster of 8 CTAs owns one probe at a time: a 256 x 256 complex64 wave (512 KB)
// is split by rows (ix) over the 8 CTAs' shared memory, 32 lines (64 KB) each,
// and stays there from the first slice to the detector.  Per slice
// (mulslice.cpp:706-739):
//   A  each CTA transforms its own 32 lines along iy: ifft_y, * t, fft_y
//      (half-warp lines, the two-stage radix 16 x 16 plan of the streaming
//      row pass), in place in its shared memory;            cluster barrier
//   B  each CTA gathers its 32 columns (iy) from all 8 CTAs' shared memory
//      through distributed shared memory straight into registers, in the
//      column transform's natural order;                    cluster arrive
//      fft_x, propagator and band limit, [detector sums at a checkpoint],
//      ifft_x (exchange space: the CTA's own 64 KB column area);
//                                                           cluster wait
//   C  the columns are scattered back into the owners' row lines;
//                                                           cluster barrier
// so the wave's only HBM traffic is the probe read once and the transmission
// rows (8 N^2 bytes per slice, shared through L2 by every cluster on the same
// slice).  Row lines sit in shared memory with slot iy ^ (ix & 15), which keeps
// the half-warp's 16 remote 8-byte accesses of phase B / C on 16 distinct bank
// pairs.  Detector sums: FP64 per thread, per warp, per CTA, in a fixed order;
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
constexpr size_t kOffR = 0;                                        // 32 row lines (64 KB)
constexpr size_t kOffS = kOffR + kLines * kLineBytes;              // 32 column exchange areas (64 KB)
constexpr size_t kOffTw = kOffS + kLines * kLineBytes;             // 16 x 16 stage-1 table
constexpr size_t kOffRed = kOffTw + sizeof(float2) * 256;          // per-warp detector sums
constexpr size_t kResidentSmem = kOffRed + sizeof(double) * (kThreads / 32) * kMaxDetR + kLineBytes;

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
__device__ __forceinline__ float2 ld_cluster(uint32_t addr) {
    float2 v;
    asm volatile("ld.shared::cluster.v2.f32 {%0, %1}, [%2];" : "=f"(v.x), "=f"(v.y) : "r"(addr) : "memory");
    return v;
}
__device__ __forceinline__ void st_cluster(uint32_t addr, float2 v) {
    asm volatile("st.shared::cluster.v2.f32 [%0], {%1, %2};" ::"r"(addr), "f"(v.x), "f"(v.y) : "memory");
}
// slot of (local row r, column iy) in the row lines
__device__ __forceinline__ uint32_t rslot(int r, int iy) { return (uint32_t)(r * kN + (iy ^ (r & 15))); }

}  // namespace

__global__ void __launch_bounds__(kThreads, 1) stem_resident_kernel(ResidentArgs a) {
    extern __shared__ unsigned char smraw[];
    const uint32_t AL = (uint32_t)kLineBytes;
    unsigned char *base = smraw + ((AL - (smem_u32(smraw) & (AL - 1u))) & (AL - 1u));
    float2 *R = reinterpret_cast<float2 *>(base + kOffR);
    float2 *S = reinterpret_cast<float2 *>(base + kOffS);
    float2 *tw = reinterpret_cast<float2 *>(base + kOffTw);
    double *red = reinterpret_cast<double *>(base + kOffRed);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, t = lane & 15;
    const int j = 2 * warp + (lane >> 4);  // this half-warp's row line / column (0..31)
    const uint32_t rank = cluster_rank();
    for (int i = tid; i < 256; i += kThreads) {
        float sn, cn;
        sincospif((float)(2 * (i / 16) * (i % 16)) / (float)kN, &sn, &cn);  // exp(2 pi i r k / N), [r][k]
        tw[i] = make_float2(cn, sn);
    }
    __syncthreads();
    const uint32_t Rs = smem_u32(R);
    const int ix_row = (int)rank * kLines + j;   // phase A: this half-warp's line
    const int iy_col = (int)rank * kLines + j;   // phase B: this half-warp's column
    const RowXorLin<RP> adR{Rs + (uint32_t)(j * kLineBytes)};
    const RowXorLin<RP> adS{smem_u32(S) + (uint32_t)(j * kLineBytes)};
    // remote addresses of this thread's 16 column elements: ix = t + 16 e,
    // owner rank e >> 1, local row t + 16 (e & 1)
    uint32_t raddr[RP::E];
#pragma unroll
    for (int e = 0; e < RP::E; ++e) {
        const int r = t + 16 * (e & 1);
        raddr[e] = map_rank(Rs + 8u * rslot(r, iy_col), (uint32_t)(e >> 1));
    }
    const float ky2 = a.ky2[iy_col];
    for (int b = (int)cluster_id_x(); b < a.nprobe; b += (int)nclusters_x()) {
        int ic = 0;
        for (int s = 0; s < a.nslice; ++s) {
            const int l = a.layer_seq[s];
            // ---- A: the row line ix_row
            float2 v[RP::E];
            if (s == 0) {
                const float2 *src = a.w0 + ((size_t)b * kN + ix_row) * kN;
#pragma unroll
                for (int e = 0; e < RP::E; ++e) v[e] = src[t + 16 * e];
            } else {
#pragma unroll
                for (int e = 0; e < RP::E; ++e) v[e] = R[rslot(j, t + 16 * e)];
            }
            fft_line_tab<RP, -1>(v, t, adR, tw);
            const float2 *trow = a.trans + ((size_t)l * kN + ix_row) * kN;
#pragma unroll
            for (int e = 0; e < RP::E; ++e) v[e] = c_mul(v[e], __ldg(trow + t + 16 * e));
            fft_line_tab<RP, +1>(v, t, adR, tw);
            __syncwarp();  // every lane is done with the exchange slots
#pragma unroll
            for (int e = 0; e < RP::E; ++e) R[rslot(j, t + 16 * e)] = v[e];
            cluster_arrive();
            cluster_wait();
            // ---- B: the column iy_col, gathered from the 8 CTAs
#pragma unroll
            for (int e = 0; e < RP::E; ++e) v[e] = ld_cluster(raddr[e]);
            cluster_arrive();  // this CTA's reads of the cluster's rows are issued and complete
            fft_line_tab<RP, +1>(v, t, adS, tw);
            const float2 *px = a.prop + (size_t)l * 2 * kN, *py = px + kN;
            const float2 pyv = __ldg(py + iy_col);
#pragma unroll
            for (int e = 0; e < RP::E; ++e) {
                const int ix = t + 16 * e;
                const float k2 = a.kx2[ix] + ky2;
                v[e] = k2 < a.k2max ? c_mul(c_mul(v[e], pyv), __ldg(px + ix)) : make_float2(0.f, 0.f);
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
                for (int d = 0; d < a.ndet; ++d) {
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
                __syncthreads();
                ++ic;
            }
            const bool last = s == a.nslice - 1 || ic >= a.ncheck;
            if (!last) fft_line_tab<RP, -1>(v, t, adS, tw);
            cluster_wait();  // every CTA has gathered: the row lines may be overwritten
            if (last) break;
            // ---- C: scatter back into the owners' row lines
#pragma unroll
            for (int e = 0; e < RP::E; ++e) st_cluster(raddr[e], v[e]);
            cluster_arrive();
            cluster_wait();
        }
    }
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
