// msl_multislice_noalloc: the CTEM slice loop for callers that cannot allocate
// device memory.
//
// Who needs it: a caller embedded in a host application that has already
// claimed the GPU's memory for its own pool (and forbids anyone else from
// calling cudaMalloc), or one running a latency-critical loop where a device
// allocation or free would stall every stream on the device.  Such a caller
// owns all the big buffers (transmission functions, waves) and needs the
// library to bring nothing of its own.
//
// What it does: exactly the slice loop of msl_multislice (same kernels, same
// launch sequence), but the small tables that loop reads besides its inputs
// and outputs -- twiddles of both line transforms, the float k^2 tables of the
// band limit and the per-layer propagator tables -- live in one file-scope
// device array of fixed size instead of context buffers.  No cudaMalloc,
// cudaFree or other allocating routine is called, and no context is needed.
//
// Limits: nx, ny <= 2048 (every supported side) and at most 64 layers; the
// array is 2,150,656 bytes and every GPU that loads the library holds it until
// the process exits.
//
// Sharing: every call uses the same array and leaves its tables in it.  The
// tables are rewritten in full at the start of each call, on the caller's
// stream, together with the error word the pass kernels raise (cleared to
// zero), and the call waits for its stream before returning; calls that
// overlap on the GPU -- from different host threads on different streams of
// one device -- race on the array.  Host-side, calls are serialised by a mutex.
//
// Set-up: the first call on each device looks up the array's device address
// with cudaGetSymbolAddress while that device is current (a host-side name of
// a __device__ array is not a device address).
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include <string.h>

#include <cmath>
#include <mutex>

#include "../../include/msl.h"
#include "msl_fft.cuh"
#include "msl_internal.h"

namespace {

constexpr int kMaxSide = MSL_NOALLOC_MAX_SIDE;
constexpr int kMaxLayers = MSL_NOALLOC_MAX_LAYERS;
constexpr int kMaxTw = 2304;  // largest per-side twiddle buffer (side 2048), float2 entries
// Layout of the array: the kernels' error word, then the tables.
constexpr size_t kOffErr = 0;
constexpr size_t kOffTwRow = 256;
constexpr size_t kOffTwCol = kOffTwRow + sizeof(float2) * kMaxTw;
constexpr size_t kOffKx2 = kOffTwCol + sizeof(float2) * kMaxTw;
constexpr size_t kOffKy2 = kOffKx2 + sizeof(float) * kMaxSide;
constexpr size_t kOffProp = kOffKy2 + sizeof(float) * kMaxSide;
constexpr size_t kScratchBytes = kOffProp + sizeof(float2) * (size_t)kMaxLayers * 2 * kMaxSide;
static_assert(kScratchBytes == MSL_NOALLOC_SCRATCH_BYTES, "scratch size must match msl.h");
// every side's twiddle buffer (with the two-stage 1024 row table appended) fits its slot
#define X(N) static_assert(msl::plan_tw_size<msl::Plan<N>>() <= kMaxTw, "twiddle slot too small for side " #N);
MSL_FOR_EACH_SIDE(X)
#undef X
static_assert(msl::WarpPlan1024x2::GTW_OFF + 32 * 32 <= kMaxTw, "the 1024 buffer holds the two-stage row table");
static_assert(kOffTwCol % 256 == 0 && kOffKx2 % 256 == 0 && kOffProp % 256 == 0, "alignment");

std::mutex g_mu;
unsigned char *g_dev_ptr[256] = {};                                  // per device ordinal
alignas(256) unsigned char g_host_stage[kScratchBytes];              // host copy of the tables
float g_kx[kMaxSide], g_ky[kMaxSide];                                 // float frequencies (host)

bool is_dev(const void *p, int dev) {
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return (at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged) && at.device == dev;
}

}  // namespace

// The tables' home on every device that loads the library.
static __device__ __align__(256) unsigned char g_msl_noalloc_scratch[kScratchBytes];

extern "C" int msl_multislice_noalloc(const msl_grid *g, const msl_optics *o, const float *trans,
                                      int ntrans, const double *dz, const int *layer_seq,
                                      int nslice, float *psi, int batch, int plane_wave,
                                      void *stream) {
    // ---- argument checks (all before touching the device)
    if (!g || !o || !trans || !psi || !dz || !layer_seq) return MSL_E_ARG;
    if (!msl::plan_supported(g->nx) || !msl::plan_supported(g->ny)) return MSL_E_UNSUPPORTED;
    if (g->nx > kMaxSide || g->ny > kMaxSide) return MSL_E_UNSUPPORTED;
    if (!(g->ax > 0) || !(g->by > 0) || !std::isfinite(g->ax) || !std::isfinite(g->by)) return MSL_E_ARG;
    if (!(o->kev > 0) || !std::isfinite(o->kev) || !(o->bandlimit > 0) || o->bandlimit > 1.0 ||
        !std::isfinite(o->tilt_x) || !std::isfinite(o->tilt_y))
        return MSL_E_ARG;
    if (ntrans < 1 || ntrans > kMaxLayers) return MSL_E_ARG;  // beyond the array's capacity
    if (nslice < 1 || batch < 1) return MSL_E_ARG;
    for (int l = 0; l < ntrans; ++l)
        if (!(dz[l] > 0) || !std::isfinite(dz[l])) return MSL_E_ARG;
    for (int s = 0; s < nslice; ++s)
        if (layer_seq[s] < 0 || layer_seq[s] >= ntrans) return MSL_E_ARG;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 256) return MSL_E_CUDA;
    if (!is_dev(trans, dev) || !is_dev(psi, dev)) return MSL_E_ARG;  // caller-owned device buffers only
    cudaStream_t st = (cudaStream_t)stream;

    std::lock_guard<std::mutex> lock(g_mu);
    // ---- one-time set-up on this device: the array's device address
    if (!g_dev_ptr[dev]) {
        void *p = nullptr;
        if (cudaGetSymbolAddress(&p, g_msl_noalloc_scratch) != cudaSuccess || !p) {
            cudaGetLastError();
            return MSL_E_CUDA;
        }
        g_dev_ptr[dev] = (unsigned char *)p;
    }
    unsigned char *d = g_dev_ptr[dev];
    const int nx = g->nx, ny = g->ny;
    int nsm = 1;
    if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return MSL_E_CUDA;

    // ---- tables, built on the host by the same helpers msl_multislice uses
    float2 *h_twr = (float2 *)(g_host_stage + kOffTwRow), *h_twc = (float2 *)(g_host_stage + kOffTwCol);
    float *h_kx2 = (float *)(g_host_stage + kOffKx2), *h_ky2 = (float *)(g_host_stage + kOffKy2);
    float2 *h_prop = (float2 *)(g_host_stage + kOffProp);
    *(int *)(g_host_stage + kOffErr) = 0;  // the error word starts every call at zero
    if (msl::plan_twiddles_into(ny, h_twr, kMaxTw) < 0 || msl::plan_twiddles_into(nx, h_twc, kMaxTw) < 0)
        return MSL_E_UNSUPPORTED;
    msl::freqn_f32(nx, g->ax, g_kx, h_kx2);
    msl::freqn_f32(ny, g->by, g_ky, h_ky2);
    const float k2max = msl::k2max_f32(nx, ny, g->ax, g->by, o->bandlimit);
    for (int l = 0; l < ntrans; ++l) {
        float2 *px = h_prop + (size_t)l * (nx + ny), *py = px + nx;
        msl::prop_tables(nx, ny, o, dz[l], g_kx, h_kx2, g_ky, h_ky2, px, py);
    }
    // ---- into the device array (every region this call reads is rewritten)
    const size_t prop_bytes = sizeof(float2) * (size_t)ntrans * (nx + ny);
    if (cudaMemcpyAsync(d, g_host_stage, kOffProp + prop_bytes, cudaMemcpyHostToDevice, st) != cudaSuccess)
        return MSL_E_CUDA;
    int *derr = (int *)(d + kOffErr);
    // a failure after the upload still waits for what is queued, so no kernel of
    // this call reads the array once the lock is released
    auto bail = [&]() {
        cudaStreamSynchronize(st);
        cudaGetLastError();
        return MSL_E_CUDA;
    };

    // ---- the slice loop of msl_multislice
    const float2 *twr = (const float2 *)(d + kOffTwRow), *twc = (const float2 *)(d + kOffTwCol);
    const float *kx2d = (const float *)(d + kOffKx2), *ky2d = (const float *)(d + kOffKy2);
    const float2 *propd = (const float2 *)(d + kOffProp);
    float2 *w = (float2 *)psi;
    const float2 *td = (const float2 *)trans;
    const size_t n2 = (size_t)nx * ny;
    int64_t launches = 0;
    auto row = [&](const float2 *tr, int flags) {
        msl::RowArgs a;
        memset(&a, 0, sizeof(a));
        a.in = w;
        a.out = w;
        a.nlines = batch * nx;
        a.nx = nx;
        a.trans = tr;
        a.tw = twr;
        a.flags = flags;
        a.scale = 1.0f;
        a.err = derr;
        return msl::launch_row_pass(ny, a, st, nsm, &launches);
    };
    auto col = [&](int layer) {
        msl::ColArgs a;
        memset(&a, 0, sizeof(a));
        a.in = w;
        a.out = w;
        a.batch = batch;
        a.ny = ny;
        a.tw = twc;
        a.flags = msl::COL_LOAD | msl::COL_FWD | msl::COL_PROP | msl::COL_INV | msl::COL_STORE;
        a.px = propd + (size_t)layer * (nx + ny);
        a.py = a.px + nx;
        a.kx2 = kx2d;
        a.ky2 = ky2d;
        a.k2max = k2max;
        a.err = derr;
        return msl::launch_col_pass(nx, a, st, nsm, &launches);
    };
    for (int s = 0; s < nslice; ++s) {
        const int l = layer_seq[s];
        int rf = msl::ROW_TRANS | msl::ROW_FWD;
        if (s > 0) rf |= msl::ROW_LOAD | msl::ROW_INV;
        else if (!plane_wave) rf |= msl::ROW_LOAD;
        if (row(td + (size_t)l * n2, rf) != cudaSuccess) return bail();
        if (col(l) != cudaSuccess) return bail();
    }
    if (row(nullptr, msl::ROW_LOAD | msl::ROW_INV) != cudaSuccess) return bail();
    // the error word: 1 = a pass's bounded wait gave up, 2 = a pass found its
    // aligned slots outside its shared memory; either leaves the wave partly
    // transformed.  A pageable copy into a host int allocates nothing.
    int herr = 0;
    if (cudaMemcpyAsync(&herr, derr, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess) return bail();
    if (cudaStreamSynchronize(st) != cudaSuccess) return MSL_E_CUDA;
    if (herr) return MSL_E_CUDA;
    return MSL_OK;
}
