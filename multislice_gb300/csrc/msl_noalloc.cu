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
// array is 2,150,400 bytes and every GPU that loads the library holds it until
// the process exits.
//
// Sharing: every call uses the same array and leaves its tables in it.  The
// tables are rewritten in full at the start of each call (nothing is expected
// to start at zero), on the caller's stream, and the call waits for its stream
// before returning; calls that overlap on the GPU -- from different host
// threads on different streams of one device -- race on the array.  Host-side,
// calls are serialised by a mutex.
//
// Set-up: the first call on each device looks up the array's device address
// with cudaGetSymbolAddress while that device is current (a host-side name of
// a __device__ array is not a device address).  Make that first call before
// any stream capture begins.
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
constexpr size_t kOffTwRow = 0;
constexpr size_t kOffTwCol = kOffTwRow + sizeof(float2) * kMaxTw;
constexpr size_t kOffKx2 = kOffTwCol + sizeof(float2) * kMaxTw;
constexpr size_t kOffKy2 = kOffKx2 + sizeof(float) * kMaxSide;
constexpr size_t kOffProp = kOffKy2 + sizeof(float) * kMaxSide;
constexpr size_t kScratchBytes = kOffProp + sizeof(float2) * (size_t)kMaxLayers * 2 * kMaxSide;
static_assert(kScratchBytes == MSL_NOALLOC_SCRATCH_BYTES, "scratch size must match msl.h");
static_assert(msl::WarpPlan1024x2::GTW_OFF + 32 * 32 <= kMaxTw, "the 1024 buffer holds the two-stage row table");
static_assert(kOffTwCol % 256 == 0 && kOffKx2 % 256 == 0 && kOffProp % 256 == 0, "alignment");

std::mutex g_mu;
unsigned char *g_dev_ptr[256] = {};                                  // per device ordinal
alignas(256) unsigned char g_host_stage[kScratchBytes];              // host copy of the tables

template <int N> void twiddles_into(float2 *out) {
    using P = msl::Plan<N>;
    for (int s = 1; s < P::NSTAGE; ++s) {
        const int R = P::radix(s), NS = msl::plan_span<P>(s), off = msl::plan_tw_offset<P>(s);
        for (int r = 0; r < R; ++r)
            for (int k = 0; k < NS; ++k) {
                const long m = ((long)r * k) % ((long)NS * R);
                const double ang = 2.0 * 3.14159265358979323846 * (double)m / (double)(NS * R);
                out[off + r * NS + k] = make_float2((float)cos(ang), (float)sin(ang));
            }
    }
}

bool twiddles_for_side(int n, float2 *out) {
    switch (n) {
        case 64: twiddles_into<64>(out); return true;
        case 128: twiddles_into<128>(out); return true;
        case 256: twiddles_into<256>(out); return true;
        case 384: twiddles_into<384>(out); return true;
        case 512: twiddles_into<512>(out); return true;
        case 768: twiddles_into<768>(out); return true;
        case 1024:
            twiddles_into<1024>(out);
            msl::append_row_two_twiddles(1024, out);  // the two-stage row kernel's table
            return true;
        case 2048: twiddles_into<2048>(out); return true;
        default: return false;
    }
}

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

    // ---- tables, built on the host exactly as msl_multislice builds them
    float2 *h_twr = (float2 *)(g_host_stage + kOffTwRow), *h_twc = (float2 *)(g_host_stage + kOffTwCol);
    float *h_kx2 = (float *)(g_host_stage + kOffKx2), *h_ky2 = (float *)(g_host_stage + kOffKy2);
    float2 *h_prop = (float2 *)(g_host_stage + kOffProp);
    if (!twiddles_for_side(ny, h_twr) || !twiddles_for_side(nx, h_twc)) return MSL_E_UNSUPPORTED;
    static float kx[kMaxSide], ky[kMaxSide];
    // spatial frequencies in float as freqn() (slicelib.cpp:433-463)
    const int imx = (int)(nx / 2.0 + 0.5), imy = (int)(ny / 2.0 + 0.5);
    for (int i = 0; i < nx; ++i) {
        kx[i] = (float)(i > imx ? i - nx : i) / (float)g->ax;
        h_kx2[i] = kx[i] * kx[i];
    }
    for (int i = 0; i < ny; ++i) {
        ky[i] = (float)(i > imy ? i - ny : i) / (float)g->by;
        h_ky2[i] = ky[i] * ky[i];
    }
    // band limit in float (mulslice.cpp:481-489)
    float k2max = (float)nx / (2.0F * (float)g->ax);
    const float tk = (float)ny / (2.0F * (float)g->by);
    if (tk < k2max) k2max = tk;
    k2max = (float)o->bandlimit * k2max;
    k2max = k2max * k2max;
    // propagator tables per layer (mulslice.cpp:494-513), py carrying 1/(nx ny)
    const float scale = 1.0f / ((float)nx * (float)ny);
    const double lam = msl_wavelength(o->kev);
    for (int l = 0; l < ntrans; ++l) {
        float2 *px = h_prop + (size_t)l * (nx + ny), *py = px + nx;
        if (o->f32_prop_args) {
            const float wl = (float)lam, sc = (float)(4.0 * atan(1.0)) * (float)dz[l];
            const float tx = (float)(2.0 * tan(o->tilt_x)), ty = (float)(2.0 * tan(o->tilt_y));
            for (int i = 0; i < nx; ++i) {
                const double t = sc * (h_kx2[i] * wl - kx[i] * tx);
                px[i] = make_float2((float)cos(t), (float)-sin(t));
            }
            for (int i = 0; i < ny; ++i) {
                const double t = sc * (h_ky2[i] * wl - ky[i] * ty);
                py[i] = make_float2((float)cos(t) * scale, (float)-sin(t) * scale);
            }
        } else {
            const double pi = 3.14159265358979323846;
            const double ttx = 2.0 * tan(o->tilt_x), tty = 2.0 * tan(o->tilt_y);
            for (int i = 0; i < nx; ++i) {
                const double k = kx[i], t = pi * dz[l] * (k * k * lam - k * ttx);
                px[i] = make_float2((float)cos(t), (float)-sin(t));
            }
            for (int i = 0; i < ny; ++i) {
                const double k = ky[i], t = pi * dz[l] * (k * k * lam - k * tty);
                py[i] = make_float2((float)cos(t) * scale, (float)-sin(t) * scale);
            }
        }
    }
    // ---- into the device array (every region this call reads is rewritten)
    const size_t prop_bytes = sizeof(float2) * (size_t)ntrans * (nx + ny);
    if (cudaMemcpyAsync(d, g_host_stage, kOffProp + prop_bytes, cudaMemcpyHostToDevice, st) != cudaSuccess)
        return MSL_E_CUDA;

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
        return msl::launch_col_pass(nx, a, st, nsm, &launches);
    };
    for (int s = 0; s < nslice; ++s) {
        const int l = layer_seq[s];
        int rf = msl::ROW_TRANS | msl::ROW_FWD;
        if (s > 0) rf |= msl::ROW_LOAD | msl::ROW_INV;
        else if (!plane_wave) rf |= msl::ROW_LOAD;
        if (row(td + (size_t)l * n2, rf) != cudaSuccess) return MSL_E_CUDA;
        if (col(l) != cudaSuccess) return MSL_E_CUDA;
    }
    if (row(nullptr, msl::ROW_LOAD | msl::ROW_INV) != cudaSuccess) return MSL_E_CUDA;
    if (cudaStreamSynchronize(st) != cudaSuccess) return MSL_E_CUDA;
    return MSL_OK;
}
