// C ABI of libmsl.so: validation, buffer staging and pass sequencing on the host.
// Kernels live in msl_passes.cu and msl_potential.cu; the ABI is declared in
// include/msl.h.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <map>
#include <string>
#include <vector>

#include "../../include/msl.h"
#include "msl_internal.h"

using msl::ColArgs;
using msl::RowArgs;

namespace msl {

// Spatial frequencies in float exactly as freqn() (slicelib.cpp:433-463).
void freqn_f32(int n, double a, float *k, float *k2) {
    const int imid = (int)(n / 2.0 + 0.5);
    for (int i = 0; i < n; ++i) {
        const float num = (float)(i > imid ? i - n : i);
        k[i] = num / (float)a;
        k2[i] = k[i] * k[i];
    }
}

// Squared band limit in float as mulslice.cpp:481-489.
float k2max_f32(int nx, int ny, double ax, double by, double bw) {
    float k = (float)nx / (2.0F * (float)ax);
    float t = (float)ny / (2.0F * (float)by);
    if (t < k) k = t;
    k = (float)bw * k;
    return k * k;
}

// Propagator tables of one slice thickness (mulslice.cpp:494-513): px, py with
// py already carrying the ifft scale 1/(nx ny).
void prop_tables(int nx, int ny, const msl_optics *o, double dz, const float *kx, const float *kx2,
                 const float *ky, const float *ky2, float2 *px, float2 *py) {
    const float scale = 1.0f / ((float)nx * (float)ny);
    const double lam = msl_wavelength(o->kev);
    if (o->f32_prop_args) {
        const float wl = (float)lam;
        const float sc = (float)(4.0 * atan(1.0)) * (float)dz;
        const float tctx = (float)(2.0 * tan(o->tilt_x)), tcty = (float)(2.0 * tan(o->tilt_y));
        for (int i = 0; i < nx; ++i) {
            const double t = sc * (kx2[i] * wl - kx[i] * tctx);
            px[i] = make_float2((float)cos(t), (float)-sin(t));
        }
        for (int i = 0; i < ny; ++i) {
            const double t = sc * (ky2[i] * wl - ky[i] * tcty);
            py[i] = make_float2((float)cos(t) * scale, (float)-sin(t) * scale);
        }
        return;
    }
    const double pi = 3.14159265358979323846;
    const double ttx = 2.0 * tan(o->tilt_x), tty = 2.0 * tan(o->tilt_y);
    for (int i = 0; i < nx; ++i) {
        const double k = kx[i];
        const double t = pi * dz * (k * k * lam - k * ttx);
        px[i] = make_float2((float)cos(t), (float)-sin(t));
    }
    for (int i = 0; i < ny; ++i) {
        const double k = ky[i];
        const double t = pi * dz * (k * k * lam - k * tty);
        py[i] = make_float2((float)cos(t) * scale, (float)-sin(t) * scale);
    }
}

}  // namespace msl

namespace {

const char kVersion[] = "msl 0.1 (sm_103a)";

// Device memory held by a context's work buffers, against an optional cap
// (msl_set_memory_limit).
struct MemBudget {
    size_t limit = 0;  // 0: no cap
    size_t used = 0;
};

struct DevBuf {
    void *p = nullptr;
    size_t cap = 0;
    MemBudget *mb = nullptr;
    DevBuf() = default;
    DevBuf(const DevBuf &) = delete;
    DevBuf &operator=(const DevBuf &) = delete;
    ~DevBuf() { release(); }
    // Grow to at least `bytes`; a growth the context's cap would not allow fails
    // before anything is freed or allocated.
    cudaError_t ensure(size_t bytes) {
        if (bytes <= cap) return cudaSuccess;
        if (mb && mb->limit && mb->used - cap + bytes > mb->limit) return cudaErrorMemoryAllocation;
        release();
        cudaError_t e = cudaMalloc(&p, bytes ? bytes : 1);
        if (e == cudaSuccess) {
            cap = bytes;
            if (mb) mb->used += bytes;
        } else {
            p = nullptr;
        }
        return e;
    }
    void release() {
        if (p) cudaFree(p);
        if (mb) mb->used -= cap;
        p = nullptr;
        cap = 0;
    }
};

}  // namespace

struct msl_ctx {
    int device = 0;
    int nsm = 1;
    cudaStream_t stream = nullptr;
    std::string err;
    int64_t launches = 0;
    int probe_batch = 0;
    std::map<int, float2 *> tw;
    // optional per-kernel-kind timing with events on the context's stream
    bool prof = false;
    bool autotune = false;  // tune each side's pass families on first use (per device)
    std::vector<cudaEvent_t> ev_free;
    struct Pending { int kind; cudaEvent_t a, b; };
    std::vector<Pending> pending;
    int64_t prof_count[MSL_PROF_KINDS] = {0};
    double prof_ms[MSL_PROF_KINDS] = {0};
    MemBudget mem;
    DevBuf wave, in_stage, trans_stage, tabs, apchi, exy, fxy, detmask, partial, detout, pot,
        atoms, tmpw, ctf, acc, jobtab;
    int *dflag = nullptr;  // device flag raised by a kernel whose bounded wait gave up
    std::vector<cudaStream_t> side_streams;  // one per grid group of an uneven batch
    // msl_multislice's launch sequence for small batches, replayed as one CUDA
    // graph: the key holds every launch argument of the loop (pointers, flags,
    // schedules, the layer sequence); a key seen twice in a row is captured,
    // then replayed while it repeats
    struct LoopGraph {
        std::vector<unsigned char> seen, key;
        cudaGraphExec_t exec = nullptr;
        int64_t nlaunch = 0;
    } loop_graph;
    msl_ctx() {
        DevBuf *bufs[] = {&wave, &in_stage, &trans_stage, &tabs, &apchi, &exy, &fxy, &detmask,
                          &partial, &detout, &pot, &atoms, &tmpw, &ctf, &acc, &jobtab};
        for (DevBuf *b : bufs) b->mb = &mem;
    }
};

namespace {

int fail(msl_ctx *c, int code, const std::string &msg) {
    if (c) c->err = msg;
    return code;
}

cudaEvent_t take_event(msl_ctx *c) {
    if (!c->ev_free.empty()) {
        cudaEvent_t e = c->ev_free.back();
        c->ev_free.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    cudaEventCreate(&e);
    return e;
}

// Bracket one launch with events when profiling is on.
template <class F> cudaError_t timed(msl_ctx *c, int kind, F &&launch) {
    if (!c->prof) return launch();
    cudaEvent_t a = take_event(c), b = take_event(c);
    cudaEventRecord(a, c->stream);
    cudaError_t e = launch();
    cudaEventRecord(b, c->stream);
    c->pending.push_back({kind, a, b});
    return e;
}

// Fold finished launch timings into the per-kind totals (stream is synchronized).
void collect_profile(msl_ctx *c) {
    for (auto &p : c->pending) {
        float ms = 0.f;
        if (cudaEventElapsedTime(&ms, p.a, p.b) == cudaSuccess) {
            c->prof_count[p.kind] += 1;
            c->prof_ms[p.kind] += ms;
        }
        c->ev_free.push_back(p.a);
        c->ev_free.push_back(p.b);
    }
    c->pending.clear();
}

#define CUDA_TRY(ctx, call)                                                                  \
    do {                                                                                     \
        cudaError_t e_ = (call);                                                             \
        if (e_ != cudaSuccess)                                                               \
            return fail(ctx, e_ == cudaErrorMemoryAllocation ? MSL_E_NOMEM : MSL_E_CUDA,      \
                        std::string(#call) + ": " + cudaGetErrorString(e_));                \
    } while (0)

bool on_device(const void *p) {
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged;
}

bool is_fin(double x) { return std::isfinite(x); }

int check_grid(msl_ctx *c, const msl_grid *g) {
    if (!g) return fail(c, MSL_E_ARG, "grid is null");
    if (!msl::plan_supported(g->nx) || !msl::plan_supported(g->ny))
        return fail(c, MSL_E_UNSUPPORTED,
                    "grid side not supported (64,128,256,384,512,768,1024,2048): " +
                        std::to_string(g->nx) + "x" + std::to_string(g->ny));
    if (!(g->ax > 0) || !(g->by > 0) || !is_fin(g->ax) || !is_fin(g->by))
        return fail(c, MSL_E_ARG, "cell size must be positive and finite");
    return MSL_OK;
}

int check_optics(msl_ctx *c, const msl_optics *o) {
    if (!o) return fail(c, MSL_E_ARG, "optics is null");
    if (!(o->kev > 0) || !is_fin(o->kev)) return fail(c, MSL_E_ARG, "beam energy must be positive");
    if (!(o->bandlimit > 0) || o->bandlimit > 1.0)
        return fail(c, MSL_E_ARG, "bandlimit must lie in (0, 1]");
    if (!is_fin(o->tilt_x) || !is_fin(o->tilt_y)) return fail(c, MSL_E_ARG, "tilt must be finite");
    return MSL_OK;
}

void freqn_f32(int n, double a, std::vector<float> &k, std::vector<float> &k2) {
    k.resize(n);
    k2.resize(n);
    msl::freqn_f32(n, a, k.data(), k2.data());
}
using msl::k2max_f32;
void prop_tables(int nx, int ny, double ax, double by, const msl_optics *o, double dz,
                 const std::vector<float> &kx, const std::vector<float> &kx2,
                 const std::vector<float> &ky, const std::vector<float> &ky2, float2 *px,
                 float2 *py) {
    msl::prop_tables(nx, ny, o, dz, kx.data(), kx2.data(), ky.data(), ky2.data(), px, py);
}

float2 *twiddles(msl_ctx *c, int n) {
    auto it = c->tw.find(n);
    if (it != c->tw.end()) return it->second;
    std::vector<float2> h;
    msl::plan_twiddles(n, h);
    float2 *d = nullptr;
    if (cudaMalloc(&d, h.size() * sizeof(float2)) != cudaSuccess) return nullptr;
    if (cudaMemcpy(d, h.data(), h.size() * sizeof(float2), cudaMemcpyHostToDevice) != cudaSuccess) {
        cudaFree(d);
        return nullptr;
    }
    c->tw[n] = d;
    return d;
}

// Device view of a caller buffer: the pointer itself if it is device memory,
// else a staging buffer (copied in when `copy_in`).
template <class T>
int stage_in(msl_ctx *c, const T *p, size_t bytes, DevBuf &st, const T **out, bool copy_in = true) {
    if (on_device(p)) {
        *out = p;
        return MSL_OK;
    }
    CUDA_TRY(c, st.ensure(bytes));
    if (copy_in) CUDA_TRY(c, cudaMemcpyAsync(st.p, p, bytes, cudaMemcpyHostToDevice, c->stream));
    *out = (const T *)st.p;
    return MSL_OK;
}

int upload(msl_ctx *c, DevBuf &b, const void *h, size_t bytes) {
    CUDA_TRY(c, b.ensure(bytes));
    CUDA_TRY(c, cudaMemcpyAsync(b.p, h, bytes, cudaMemcpyHostToDevice, c->stream));
    return MSL_OK;
}

struct SliceTables {
    std::vector<float> kx, kx2, ky, ky2;
    float k2max;
    // device layout: kx2[nx] ky2[ny] kx[nx] ky[ny] | px py per layer
    float *d_kx2, *d_ky2, *d_kx = nullptr, *d_ky = nullptr;
    float2 *d_prop;  // [ntrans][nx + ny]
};

int build_slice_tables(msl_ctx *c, const msl_grid *g, const msl_optics *o, int ntrans,
                       const double *dz, SliceTables &st, DevBuf *dst = nullptr) {
    DevBuf &tb = dst ? *dst : c->tabs;
    const int nx = g->nx, ny = g->ny;
    freqn_f32(nx, g->ax, st.kx, st.kx2);
    freqn_f32(ny, g->by, st.ky, st.ky2);
    st.k2max = k2max_f32(nx, ny, g->ax, g->by, o->bandlimit);
    const size_t fbytes = ((sizeof(float) * 2 * (nx + ny) + 15) / 16) * 16;
    const size_t pbytes = sizeof(float2) * (size_t)ntrans * (nx + ny);
    std::vector<unsigned char> h(fbytes + pbytes);
    memcpy(h.data(), st.kx2.data(), sizeof(float) * nx);
    memcpy(h.data() + sizeof(float) * nx, st.ky2.data(), sizeof(float) * ny);
    memcpy(h.data() + sizeof(float) * (nx + ny), st.kx.data(), sizeof(float) * nx);
    memcpy(h.data() + sizeof(float) * (2 * nx + ny), st.ky.data(), sizeof(float) * ny);
    float2 *hp = (float2 *)(h.data() + fbytes);
    for (int l = 0; l < ntrans; ++l) {
        if (dz) {
            prop_tables(nx, ny, g->ax, g->by, o, dz[l], st.kx, st.kx2, st.ky, st.ky2,
                        hp + (size_t)l * (nx + ny), hp + (size_t)l * (nx + ny) + nx);
        } else {  // identity propagator: band limit and ifft scale only
            const float scale = 1.0f / ((float)nx * (float)ny);
            for (int i = 0; i < nx; ++i) hp[(size_t)l * (nx + ny) + i] = make_float2(1.f, 0.f);
            for (int i = 0; i < ny; ++i) hp[(size_t)l * (nx + ny) + nx + i] = make_float2(scale, 0.f);
        }
    }
    int rc = upload(c, tb, h.data(), h.size());
    if (rc) return rc;
    st.d_kx2 = (float *)tb.p;
    st.d_ky2 = st.d_kx2 + nx;
    st.d_kx = st.d_ky2 + ny;
    st.d_ky = st.d_kx + nx;
    st.d_prop = (float2 *)((unsigned char *)tb.p + fbytes);
    return MSL_OK;
}

ColArgs col_args(const msl_grid *g, const SliceTables &st, float2 *tw, int layer, float2 *wave,
                 int batch, int flags, int *err) {
    ColArgs a;
    memset(&a, 0, sizeof(a));
    a.err = err;
    a.in = wave;
    a.out = wave;
    a.batch = batch;
    a.ny = g->ny;
    a.tw = tw;
    a.flags = flags;
    a.px = st.d_prop + (size_t)layer * (g->nx + g->ny);
    a.py = a.px + g->nx;
    a.kx2 = st.d_kx2;
    a.ky2 = st.d_ky2;
    a.k2max = st.k2max;
    return a;
}

RowArgs row_args(const msl_grid *g, float2 *tw, const float2 *trans, float2 *wave, int batch,
                 int flags, int *err) {
    RowArgs a;
    memset(&a, 0, sizeof(a));
    a.err = err;
    a.in = wave;
    a.out = wave;
    a.nlines = batch * g->nx;
    a.nx = g->nx;
    a.trans = trans;
    a.tw = tw;
    a.flags = flags;
    a.scale = 1.0f;
    return a;
}

#define LAUNCH_TRY(ctx, call)                                                                \
    do {                                                                                     \
        cudaError_t e_ = (call);                                                             \
        if (e_ != cudaSuccess)                                                               \
            return fail(ctx, MSL_E_CUDA, std::string("kernel launch: ") + cudaGetErrorString(e_)); \
    } while (0)

// Zero the kernel error flag before a call's launches.
int err_reset(msl_ctx *c) {
    if (!c->dflag) {
        CUDA_TRY(c, cudaMalloc(&c->dflag, sizeof(int)));
    }
    CUDA_TRY(c, cudaMemsetAsync(c->dflag, 0, sizeof(int), c->stream));
    return MSL_OK;
}

// After the stream is synchronized: fail if a kernel raised the flag.
int err_check(msl_ctx *c) {
    int h = 0;
    CUDA_TRY(c, cudaMemcpy(&h, c->dflag, sizeof(int), cudaMemcpyDeviceToHost));
    if (h == 2) return fail(c, MSL_E_CUDA, "a pass found its aligned tile or line slots outside its shared memory");
    if (h) return fail(c, MSL_E_CUDA, "a pass's bounded wait for its bulk / TMA copy timed out");
    return MSL_OK;
}

// Runs a launch sequence on the context's stream directly, or through the
// context's cached CUDA graph: replayed when `key` equals the cached key,
// captured (then replayed) when the same key came twice in a row, else run
// directly.  A failed capture leaves the stream out of capture and the cache
// empty.
struct LoopGraphRun {
    msl_ctx *c;
    explicit LoopGraphRun(msl_ctx *c_) : c(c_) {}
    template <class F> int run(const std::vector<unsigned char> &key, F &&launches) {
        msl_ctx::LoopGraph &G = c->loop_graph;
        if (G.exec && G.key == key) {
            CUDA_TRY(c, cudaGraphLaunch(G.exec, c->stream));
            c->launches += G.nlaunch;
            return MSL_OK;
        }
        if (G.seen != key) {  // first sight: run directly, remember it
            G.seen = key;
            return launches();
        }
        if (G.exec) {
            cudaGraphExecDestroy(G.exec);
            G.exec = nullptr;
            G.key.clear();
        }
        if (cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
            cudaGetLastError();  // no capture on this stream now: launch directly
            G.seen.clear();
            return launches();
        }
        const int64_t l0 = c->launches;
        const int rc = launches();
        cudaGraph_t graph = nullptr;
        const cudaError_t e = cudaStreamEndCapture(c->stream, &graph);
        if (rc || e != cudaSuccess || !graph) {
            if (graph) cudaGraphDestroy(graph);
            cudaGetLastError();
            G.seen.clear();
            c->launches = l0;
            if (rc) return rc;
            return fail(c, MSL_E_CUDA, std::string("slice-loop graph capture: ") + cudaGetErrorString(e));
        }
        cudaGraphExec_t exec = nullptr;
        const cudaError_t ei = cudaGraphInstantiate(&exec, graph, 0);
        cudaGraphDestroy(graph);
        if (ei != cudaSuccess) {
            cudaGetLastError();
            G.seen.clear();
            c->launches = l0;
            return fail(c, MSL_E_CUDA, std::string("slice-loop graph instantiation: ") + cudaGetErrorString(ei));
        }
        G.exec = exec;
        G.key = key;
        G.nlaunch = c->launches - l0;
        CUDA_TRY(c, cudaGraphLaunch(G.exec, c->stream));
        return MSL_OK;
    }
};


int check_layers(msl_ctx *c, int ntrans, const double *dz, const int *layer_seq, int nslice) {
    if (ntrans < 1) return fail(c, MSL_E_ARG, "ntrans must be >= 1");
    if (nslice < 1) return fail(c, MSL_E_ARG, "nslice must be >= 1");
    if (!dz || !layer_seq) return fail(c, MSL_E_ARG, "dz and layer_seq are required");
    for (int l = 0; l < ntrans; ++l)
        if (!(dz[l] > 0) || !is_fin(dz[l])) return fail(c, MSL_E_ARG, "slice thickness must be positive");
    for (int s = 0; s < nslice; ++s)
        if (layer_seq[s] < 0 || layer_seq[s] >= ntrans)
            return fail(c, MSL_E_ARG, "layer_seq entry out of range at slice " + std::to_string(s));
    return MSL_OK;
}


// Slice loop plus objective-lens imaging on device buffers (mulslice.cpp:539-676
// with one illumination angle).  w: [batch][nx][ny] entrance waves (ignored when
// plane) and, on return, exit waves when want_exit; img_d / exit_d: FP64
// accumulators (exit_d may be null); ttab: optional per-image transmission
// rows, [slice step][image] device pointers (td unused then).
int ctem_core(msl_ctx *c, const msl_grid *g, const msl_optics *o, const float2 *td, int ntrans,
              const double *dz, const int *seq, int nslice, const msl_lens *lens, float2 *w,
              int batch, bool plane, double weight, double *img_d, double *exit_d, bool want_exit,
              const float2 *const *ttab) {
    int rc;
    const int nx = g->nx, ny = g->ny;
    const size_t n2 = (size_t)nx * ny;
    SliceTables st;
    if ((rc = build_slice_tables(c, g, o, ntrans, dz, st))) return rc;
    float2 *twr = twiddles(c, ny), *twc = twiddles(c, nx);
    if (!twr || !twc) return fail(c, MSL_E_NOMEM, "twiddle table allocation failed");
    for (int s = 0; s < nslice; ++s) {
        const int l = seq[s];
        int rf = msl::ROW_TRANS | msl::ROW_FWD;
        if (s > 0) rf |= msl::ROW_LOAD | msl::ROW_INV;
        else if (!plane) rf |= msl::ROW_LOAD;
        // ttab: every image its own transmission, [slice step][image] row pointers
        RowArgs r = row_args(g, twr, ttab ? nullptr : td + (size_t)l * n2, w, batch, rf, c->dflag);
        if (ttab) r.trans_b = ttab + (size_t)s * batch;
        LAUNCH_TRY(c, timed(c, MSL_PROF_ROW, [&] { return msl::launch_row_pass(ny, r, c->stream, c->nsm, &c->launches); }));
        // the last slice keeps the spectrum: W = Psi(k) / (nx ny) after the propagator
        int cf = msl::COL_LOAD | msl::COL_FWD | msl::COL_PROP | msl::COL_STORE;
        if (s + 1 < nslice) cf |= msl::COL_INV;
        ColArgs ca = col_args(g, st, twc, l, w, batch, cf, c->dflag);
        LAUNCH_TRY(c, timed(c, MSL_PROF_COL, [&] { return msl::launch_col_pass(nx, ca, c->stream, c->nsm, &c->launches); }));
    }
    const size_t ibytes = sizeof(float2) * n2;  // one image
    CUDA_TRY(c, c->tmpw.ensure(ibytes));
    float2 *tmp = (float2 *)c->tmpw.p;
    // defocus values and weights (mulslice.cpp:552, :610-642)
    std::vector<double> dfs, pw;
    if (lens->df_spread > 0) {
        const int ndf = (int)((2.5 * lens->df_spread) / lens->df_step);
        for (int j = -ndf; j <= ndf; ++j) {
            const double x = j * lens->df_step / lens->df_spread;
            dfs.push_back(lens->df + j * lens->df_step);
            pw.push_back(exp(-0.5 * x * x));
        }
    } else {
        dfs.push_back(lens->df);
        pw.push_back(1.0);
    }
    double psum = 0.0;
    for (double v : pw) psum += v;
    CUDA_TRY(c, c->ctf.ensure(sizeof(float2) * n2 * dfs.size()));
    float2 *ctf = (float2 *)c->ctf.p;
    const float kob = (float)lens->k_obj;
    msl::CtfParams cp;
    cp.lam = msl_wavelength(o->kev);
    cp.cs = lens->cs;
    cp.dfa2 = lens->dfa2;
    cp.dfa2phi = lens->dfa2phi;
    cp.dfa3 = lens->dfa3;
    cp.dfa3phi = lens->dfa3phi;
    cp.k2obj = kob * kob;
    cp.scale = 1.0f;
    for (size_t j = 0; j < dfs.size(); ++j) {
        cp.df = dfs[j];
        LAUNCH_TRY(c, timed(c, MSL_PROF_OTHER, [&] {
                       return msl::launch_ctf_table(nx, ny, st.d_kx2, st.d_ky2, st.d_kx, st.d_ky, cp,
                                                    ctf + n2 * j, c->stream, &c->launches);
                   }));
    }
    const bool exit_needed = want_exit || exit_d != nullptr;
    // every image of the batch: its spectrum W = Psi(k) / (nx ny) sits in its slot
    for (int b = 0; b < batch; ++b) {
        float2 *wb = w + (size_t)b * n2;
        for (size_t j = 0; j < dfs.size(); ++j) {
            // the last image may consume the slot itself unless the exit wave still needs it
            const bool last = j + 1 == dfs.size();
            float2 *target = (last && !exit_needed) ? wb : tmp;
            if (target != wb)
                CUDA_TRY(c, cudaMemcpyAsync(target, wb, ibytes, cudaMemcpyDeviceToDevice, c->stream));
            ColArgs ca = col_args(g, st, twc, 0, target, 1,
                                  msl::COL_LOAD | msl::COL_CTF | msl::COL_INV | msl::COL_STORE, c->dflag);
            ca.ctf = ctf + n2 * j;
            LAUNCH_TRY(c, timed(c, MSL_PROF_COL, [&] { return msl::launch_col_pass(nx, ca, c->stream, c->nsm, &c->launches); }));
            RowArgs r = row_args(g, twr, nullptr, target, 1,
                                 msl::ROW_LOAD | msl::ROW_INV | msl::ROW_ACCUM | msl::ROW_NOSTORE, c->dflag);
            r.accum = img_d;
            r.accum_w = weight * pw[j] / psum;
            LAUNCH_TRY(c, timed(c, MSL_PROF_ROW, [&] { return msl::launch_row_pass(ny, r, c->stream, c->nsm, &c->launches); }));
        }
        if (exit_needed) {  // exit wave: inverse transform of W in place
            ColArgs ca = col_args(g, st, twc, 0, wb, 1, msl::COL_LOAD | msl::COL_INV | msl::COL_STORE, c->dflag);
            LAUNCH_TRY(c, timed(c, MSL_PROF_COL, [&] { return msl::launch_col_pass(nx, ca, c->stream, c->nsm, &c->launches); }));
            int rf = msl::ROW_LOAD | msl::ROW_INV;
            if (exit_d) rf |= msl::ROW_ACCUM;
            if (!want_exit) rf |= msl::ROW_NOSTORE;
            RowArgs r = row_args(g, twr, nullptr, wb, 1, rf, c->dflag);
            r.accum = exit_d;
            r.accum_w = weight;
            LAUNCH_TRY(c, timed(c, MSL_PROF_ROW, [&] { return msl::launch_row_pass(ny, r, c->stream, c->nsm, &c->launches); }));
        }
    }
    return MSL_OK;
}

int check_lens(msl_ctx *c, const msl_lens *l) {
    if (!l) return fail(c, MSL_E_ARG, "lens is null");
    if (!is_fin(l->cs) || !is_fin(l->df) || !(l->k_obj > 0) || !is_fin(l->k_obj))
        return fail(c, MSL_E_ARG, "lens: cs, df finite and k_obj > 0 required");
    if (!is_fin(l->dfa2) || !is_fin(l->dfa2phi) || !is_fin(l->dfa3) || !is_fin(l->dfa3phi))
        return fail(c, MSL_E_ARG, "lens: astigmatism terms must be finite");
    if (!(l->df_spread >= 0) || !is_fin(l->df_spread) ||
        (l->df_spread > 0 && (!(l->df_step > 0) || 2.5 * l->df_spread / l->df_step > 1000)))
        return fail(c, MSL_E_ARG, "lens: df_spread >= 0 and df_step > 0 (at most 2001 defocus values)");
    return MSL_OK;
}

uint64_t splitmix64(uint64_t x) {
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}

}  // namespace

namespace {

// ---------------------------------------------------------------- autotuner
// Tuned sides per device (bit = side slot), shared by every context of a device.
std::atomic<uint32_t> g_tuned[64];

int side_bit(int n) {
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

// Times one slice step (the slice loop's row pass then its column pass) of
// `batch` synthetic waves of side n for every pair of pass families, `reps`
// steps after one warm-up step, with events on the context's stream; keeps the
// fastest pair as the device's schedule for side n.  ms[rf * 3 + cf] receives
// the time per step of each pair.
int tune_side(msl_ctx *c, int n, int batch, int reps, int *best_r, int *best_c, double *ms) {
    const size_t n2 = (size_t)n * n;
    if (c->mem.limit) {
        const size_t cap = c->mem.limit / 4 / (sizeof(float2) * n2);
        if ((size_t)batch > cap) batch = (int)std::max<size_t>(1, cap);
    }
    CUDA_TRY(c, c->wave.ensure(sizeof(float2) * n2 * batch));
    CUDA_TRY(c, c->trans_stage.ensure(sizeof(float2) * n2));
    CUDA_TRY(c, cudaMemsetAsync(c->wave.p, 0, sizeof(float2) * n2 * batch, c->stream));
    CUDA_TRY(c, cudaMemsetAsync(c->trans_stage.p, 0, sizeof(float2) * n2, c->stream));
    msl_grid g = {n, n, 0.1 * n, 0.1 * n};
    msl_optics o = {200.0, 2.0 / 3.0, 0.0, 0.0, 0};
    const double dz = 1.5;
    SliceTables st;
    int rc;
    if ((rc = build_slice_tables(c, &g, &o, 1, &dz, st))) return rc;
    float2 *tw = twiddles(c, n);
    if (!tw) return fail(c, MSL_E_NOMEM, "twiddle table allocation failed");
    float2 *w = (float2 *)c->wave.p;
    const float2 *t = (const float2 *)c->trans_stage.p;
    cudaEvent_t e0 = take_event(c), e1 = take_event(c);
    int prev_r = 0, prev_c = 0;
    msl::get_schedule(n, &prev_r, &prev_c);
    double best = 1e300;
    *best_r = prev_r;
    *best_c = prev_c;
    for (int rf = 0; rf < msl::FAM_COUNT; ++rf)
        for (int cf = 0; cf < msl::FAM_COUNT; ++cf) {
            msl::set_schedule(n, rf, cf);
            auto step = [&]() -> cudaError_t {
                RowArgs r = row_args(&g, tw, t, w, batch, msl::ROW_LOAD | msl::ROW_INV | msl::ROW_TRANS | msl::ROW_FWD,
                                     c->dflag);
                cudaError_t e = msl::launch_row_pass(n, r, c->stream, c->nsm, &c->launches);
                if (e != cudaSuccess) return e;
                ColArgs ca = col_args(&g, st, tw, 0, w, batch,
                                      msl::COL_LOAD | msl::COL_FWD | msl::COL_PROP | msl::COL_INV | msl::COL_STORE,
                                      c->dflag);
                return msl::launch_col_pass(n, ca, c->stream, c->nsm, &c->launches);
            };
            cudaError_t e = step();
            if (e == cudaSuccess) e = cudaEventRecord(e0, c->stream);
            for (int i = 0; i < reps && e == cudaSuccess; ++i) e = step();
            if (e == cudaSuccess) e = cudaEventRecord(e1, c->stream);
            if (e == cudaSuccess) e = cudaEventSynchronize(e1);
            float t_ms = 0.f;
            if (e == cudaSuccess) e = cudaEventElapsedTime(&t_ms, e0, e1);
            if (e != cudaSuccess) {
                msl::set_schedule(n, prev_r, prev_c);
                c->ev_free.push_back(e0);
                c->ev_free.push_back(e1);
                return fail(c, MSL_E_CUDA, std::string("autotune: ") + cudaGetErrorString(e));
            }
            const double per = (double)t_ms / reps;
            if (ms) ms[rf * msl::FAM_COUNT + cf] = per;
            if (per < best) {
                best = per;
                *best_r = rf;
                *best_c = cf;
            }
        }
    c->ev_free.push_back(e0);
    c->ev_free.push_back(e1);
    msl::set_schedule(n, *best_r, *best_c);
    if ((rc = err_check(c))) return rc;
    return MSL_OK;
}

// First use of side n on this device with autotuning on: tune it once.
int maybe_tune(msl_ctx *c, int n) {
    if (!c->autotune) return MSL_OK;
    const int b = side_bit(n);
    if (b < 0 || c->device < 0 || c->device >= 64) return MSL_OK;
    if (g_tuned[c->device].load() & (1u << b)) return MSL_OK;
    int rf, cf;
    const int batch = (int)std::max<size_t>(1, ((size_t)256 << 20) / (sizeof(float2) * (size_t)n * n));
    int rc = err_reset(c);
    if (rc) return rc;
    if ((rc = tune_side(c, n, batch, 3, &rf, &cf, nullptr))) return rc;
    g_tuned[c->device].fetch_or(1u << b);
    return MSL_OK;
}

}  // namespace

extern "C" {

const char *msl_version(void) { return kVersion; }

double msl_wavelength(double kev) {
    const double emass = 510.99906, hc = 12.3984244;
    return hc / sqrt(kev * (2.0 * emass + kev));
}

double msl_sigma(double kev) {
    const double emass = 510.99906;
    const double x = (emass + kev) / (2.0 * emass + kev);
    return 2.0 * (4.0 * atan(1.0)) * x / (msl_wavelength(kev) * kev);
}

int msl_ctx_create(int device, msl_ctx **out) {
    if (!out) return MSL_E_ARG;
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
        cudaGetLastError();
        return MSL_E_CUDA;
    }
    if (device < 0 || device >= ndev) return MSL_E_ARG;
    msl_ctx *c = new msl_ctx();
    c->device = device;
    if (cudaSetDevice(device) != cudaSuccess ||
        cudaDeviceGetAttribute(&c->nsm, cudaDevAttrMultiProcessorCount, device) != cudaSuccess ||
        cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete c;
        return MSL_E_CUDA;
    }
    *out = c;
    return MSL_OK;
}

int msl_ctx_destroy(msl_ctx *c) {
    if (!c) return MSL_E_ARG;
    cudaSetDevice(c->device);
    cudaStreamSynchronize(c->stream);
    for (auto &kv : c->tw) cudaFree(kv.second);
    DevBuf *bufs[] = {&c->wave, &c->in_stage, &c->trans_stage, &c->tabs, &c->apchi, &c->exy,
                      &c->fxy, &c->detmask, &c->partial, &c->detout, &c->pot, &c->atoms,
                      &c->tmpw, &c->ctf, &c->acc, &c->jobtab};
    for (DevBuf *b : bufs) b->release();
    if (c->dflag) cudaFree(c->dflag);
    if (c->loop_graph.exec) cudaGraphExecDestroy(c->loop_graph.exec);
    for (cudaStream_t s : c->side_streams) cudaStreamDestroy(s);
    cudaStreamDestroy(c->stream);
    delete c;
    return MSL_OK;
}

const char *msl_last_error(const msl_ctx *c) { return c ? c->err.c_str() : "null context"; }

int64_t msl_kernel_launches(const msl_ctx *c) { return c ? c->launches : 0; }

int msl_profile_enable(msl_ctx *c, int on) {
    if (!c) return MSL_E_ARG;
    c->prof = on != 0;
    for (int k = 0; k < MSL_PROF_KINDS; ++k) {
        c->prof_count[k] = 0;
        c->prof_ms[k] = 0.0;
    }
    return MSL_OK;
}

int msl_profile_read(const msl_ctx *c, int kind, int64_t *launches, double *ms) {
    if (!c || kind < 0 || kind >= MSL_PROF_KINDS || !launches || !ms) return MSL_E_ARG;
    *launches = c->prof_count[kind];
    *ms = c->prof_ms[kind];
    return MSL_OK;
}


int msl_amorphous(uint64_t seed, double bx, double by, double thickness, double density, double dmin, int nz,
                  const int *zs, const double *weights, int capacity, double *xyz, int *zout, int *count) {
    if (!(bx > 0) || !(by > 0) || !(thickness > 0) || !(density > 0) || !(dmin >= 0) || nz < 1 || !zs || !weights ||
        !count || capacity < 0 || !is_fin(bx + by + thickness + density + dmin))
        return MSL_E_ARG;
    const long target = std::lround(density * bx * by * thickness);
    if (target > capacity || (target > 0 && (!xyz || !zout))) {
        *count = (int)target;  // the capacity a call needs
        return MSL_E_ARG;
    }
    double wsum = 0.0;
    for (int i = 0; i < nz; ++i) {
        if (!(weights[i] >= 0)) return MSL_E_ARG;
        wsum += weights[i];
    }
    if (!(wsum > 0)) return MSL_E_ARG;
    // cells of side >= dmin: a conflict can only come from the 27 neighbouring cells
    const double cell = dmin > 0 ? dmin : 1.0;
    const int ncx = std::max(1, (int)(bx / cell)), ncy = std::max(1, (int)(by / cell)),
              ncz = std::max(1, (int)(thickness / cell));
    const double sx = bx / ncx, sy = by / ncy, sz = thickness / ncz;
    std::vector<std::vector<int>> grid((size_t)ncx * ncy * ncz);
    uint64_t ctr = 0;
    auto uni = [&]() { return (double)(splitmix64(seed ^ splitmix64(ctr++)) >> 11) * (1.0 / 9007199254740992.0); };
    long n = 0;
    const long max_tries = 100 * std::max<long>(target, 1);
    const double d2min = dmin * dmin;
    for (long tries = 0; n < target && tries < max_tries; ++tries) {
        const double x = uni() * bx, y = uni() * by, z = uni() * thickness;
        const int cx = std::min(ncx - 1, (int)(x / sx)), cy = std::min(ncy - 1, (int)(y / sy)),
                  cz = std::min(ncz - 1, (int)(z / sz));
        bool ok = true;
        for (int ox = -1; ox <= 1 && ok; ++ox)
            for (int oy = -1; oy <= 1 && ok; ++oy)
                for (int oz = -1; oz <= 1 && ok; ++oz) {
                    const int qz = cz + oz;
                    if (qz < 0 || qz >= ncz) continue;
                    const int qx = (cx + ox + ncx) % ncx, qy = (cy + oy + ncy) % ncy;
                    for (int a : grid[((size_t)qx * ncy + qy) * ncz + qz]) {
                        double dx = x - xyz[3 * a], dy = y - xyz[3 * a + 1];
                        const double dz = z - xyz[3 * a + 2];
                        dx -= bx * std::round(dx / bx);
                        dy -= by * std::round(dy / by);
                        if (dx * dx + dy * dy + dz * dz < d2min) {
                            ok = false;
                            break;
                        }
                    }
                }
        if (!ok) continue;
        xyz[3 * n] = x;
        xyz[3 * n + 1] = y;
        xyz[3 * n + 2] = z;
        double u = uni() * wsum;
        int k = 0;
        while (k < nz - 1 && u >= weights[k]) u -= weights[k++];
        zout[n] = zs[k];
        grid[((size_t)cx * ncy + cy) * ncz + cz].push_back((int)n);
        ++n;
    }
    *count = (int)n;
    return MSL_OK;
}

int msl_phonon_displacements(uint64_t seed, int config, int natom, double sigma, double *d) {
    if (natom < 0 || config < 0 || !(sigma >= 0) || (natom > 0 && !d)) return MSL_E_ARG;
    const double two_pi = 6.283185307179586477;
    for (int i = 0; i < natom; ++i) {
        double u[4];
        for (int k = 0; k < 4; ++k) {
            const uint64_t key = ((uint64_t)config << 40) | ((uint64_t)i << 2) | (uint64_t)k;
            const uint64_t h = splitmix64(seed ^ splitmix64(key));
            u[k] = (double)(h >> 11) * (1.0 / 9007199254740992.0);
        }
        const double r0 = sqrt(-2.0 * log(1.0 - u[0])), r1 = sqrt(-2.0 * log(1.0 - u[2]));
        d[3 * i + 0] = sigma * r0 * cos(two_pi * u[1]);
        d[3 * i + 1] = sigma * r0 * sin(two_pi * u[1]);
        d[3 * i + 2] = sigma * r1 * cos(two_pi * u[3]);
    }
    return MSL_OK;
}

int msl_ctem_image(msl_ctx *c, const msl_grid *g, const msl_optics *o, const float *trans,
                   int ntrans, const double *dz, const int *layer_seq, int nslice, const msl_lens *lens,
                   float *psi, int batch, int plane_wave, double weight, double *image,
                   double *exit_intensity) {
    if (!c) return MSL_E_ARG;
    int rc = check_grid(c, g);
    if (rc) return rc;
    if ((rc = check_optics(c, o))) return rc;
    if ((rc = check_layers(c, ntrans, dz, layer_seq, nslice))) return rc;
    if ((rc = check_lens(c, lens))) return rc;
    if (!trans || !image || batch < 1 || (!plane_wave && !psi) || !is_fin(weight))
        return fail(c, MSL_E_ARG, "trans, image required; psi required unless plane_wave; batch >= 1");
    CUDA_TRY(c, cudaSetDevice(c->device));
    if ((rc = err_reset(c))) return rc;
    const int nx = g->nx, ny = g->ny;
    const size_t n2 = (size_t)nx * ny;
    const float2 *td;
    if ((rc = stage_in(c, (const float2 *)trans, sizeof(float2) * n2 * ntrans, c->trans_stage, &td)))
        return rc;
    const size_t wbytes = sizeof(float2) * n2 * batch;
    const bool pdev = psi && on_device(psi);
    float2 *w;
    if (pdev) {
        w = (float2 *)psi;
    } else {
        CUDA_TRY(c, c->wave.ensure(wbytes));
        w = (float2 *)c->wave.p;
        if (!plane_wave) CUDA_TRY(c, cudaMemcpyAsync(w, psi, wbytes, cudaMemcpyHostToDevice, c->stream));
    }
    // FP64 accumulators: caller's device buffers, or staged copies of the host ones
    const size_t ibytes = sizeof(double) * n2;
    const bool idev = on_device(image), edev = exit_intensity && on_device(exit_intensity);
    CUDA_TRY(c, c->acc.ensure(2 * ibytes));
    double *img_d = idev ? image : (double *)c->acc.p;
    double *exit_d = exit_intensity ? (edev ? exit_intensity : (double *)c->acc.p + n2) : nullptr;
    if (!idev) CUDA_TRY(c, cudaMemcpyAsync(img_d, image, ibytes, cudaMemcpyHostToDevice, c->stream));
    if (exit_intensity && !edev)
        CUDA_TRY(c, cudaMemcpyAsync(exit_d, exit_intensity, ibytes, cudaMemcpyHostToDevice, c->stream));
    if ((rc = ctem_core(c, g, o, td, ntrans, dz, layer_seq, nslice, lens, w, batch, plane_wave != 0, weight,
                        img_d, exit_d, psi != nullptr, nullptr)))
        return rc;
    if (psi && !pdev) CUDA_TRY(c, cudaMemcpyAsync(psi, w, wbytes, cudaMemcpyDeviceToHost, c->stream));
    if (!idev) CUDA_TRY(c, cudaMemcpyAsync(image, img_d, ibytes, cudaMemcpyDeviceToHost, c->stream));
    if (exit_intensity && !edev)
        CUDA_TRY(c, cudaMemcpyAsync(exit_intensity, exit_d, ibytes, cudaMemcpyDeviceToHost, c->stream));
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    collect_profile(c);
    if (c->dflag && (rc = err_check(c))) return rc;
    return MSL_OK;
}

namespace {

// Host half of a potential build: the atoms validated and binned by slice
// (stably, so the sum order inside a slice is the input order), the
// per-species parameters and radial tables, laid out as one upload image
// off | ic | jc | fx | fy | Z | sp | xf | yf | tab | zslot.  Each atom is
// given as its nearest pixel (ic, jc) and the residue x - ic dxp, y - jc dyp
// formed in FP64 and rounded to float.  The radial tables are kept and reused
// while the species, the cutoff and the FPARAMS table stay the same.
struct PotImage {
    std::vector<unsigned char> h;
    size_t o_off = 0, o_ic = 0, o_jc = 0, o_fx = 0, o_fy = 0, o_z = 0, o_sp = 0, o_xf = 0, o_yf = 0, o_tab = 0,
           o_zs = 0;
    int nsp = 0;
    double tab_r0 = 0.15;
    std::vector<int> tab_z;
    double tab_radius = -1.0;
    const double *tab_fp = nullptr;
    std::vector<float4> tab;
};

int potential_prepare(msl_ctx *c, const msl_atoms *at, const double *fparams, const msl_grid *g, int nslice,
                      double radius, PotImage &im) {
    if (!at || !fparams) return fail(c, MSL_E_ARG, "null argument");
    if (nslice < 1) return fail(c, MSL_E_ARG, "nslice must be >= 1");
    if (!(at->cz > 0) || !is_fin(at->cz)) return fail(c, MSL_E_ARG, "thickness cz must be positive");
    if (!(radius > 0) || !(2.0 * radius < g->ax) || !(2.0 * radius < g->by))
        return fail(c, MSL_E_ARG, "cutoff radius must be positive and below half the cell");
    if (at->natom < 0 || (at->natom > 0 && (!at->x || !at->y || !at->z || !at->Z)))
        return fail(c, MSL_E_ARG, "atom arrays are required");
    const double dz = at->cz / nslice;
    std::vector<int> kz(at->natom), count(nslice + 1, 0);
    for (int i = 0; i < at->natom; ++i) {
        if (!is_fin(at->x[i]) || !is_fin(at->y[i]) || !is_fin(at->z[i]))
            return fail(c, MSL_E_ARG, "atom coordinates must be finite (atom " + std::to_string(i) + ")");
        int k = (int)std::floor(at->z[i] / dz);
        if (at->z[i] < 0.0 || k < 0 || k >= nslice) k = -1;
        if (k >= 0 && (at->Z[i] < 1 || at->Z[i] > 103))
            return fail(c, MSL_E_ARG, "atomic number out of range 1..103 (atom " + std::to_string(i) + ")");
        kz[i] = k;
        if (k >= 0) count[k + 1]++;
    }
    for (int k = 0; k < nslice; ++k) count[k + 1] += count[k];
    const int nkeep = count[nslice];
    const size_t nk = nkeep > 0 ? (size_t)nkeep : 1;
    // per-species float parameters: A = AL a, B = 2 pi sqrt(b), C = AG c / d, D = pi^2 / d
    // (constants of slicelib.cpp:2673-2674)
    bool used[104] = {false};
    for (int i = 0; i < at->natom; ++i)
        if (kz[i] >= 0) used[at->Z[i]] = true;
    const double AL = 300.8242834, AG = 150.4121417, PIK = 3.141592654;
    std::vector<float> sp(104 * 12, 0.f);
    for (int z = 1; z <= 103; ++z) {
        if (!used[z]) continue;
        const double *f = fparams + z * 12;
        for (int i = 0; i < 3; ++i) {
            const double a = f[2 * i], b = f[2 * i + 1], cc = f[6 + 2 * i], d = f[7 + 2 * i];
            if (!(b > 0) || !(d > 0) || !is_fin(a) || !is_fin(cc))
                return fail(c, MSL_E_ARG, "invalid FPARAMS row for Z=" + std::to_string(z));
            sp[z * 12 + 2 * i] = (float)(AL * a);
            sp[z * 12 + 2 * i + 1] = (float)(2.0 * PIK * sqrt(b));
            sp[z * 12 + 6 + 2 * i] = (float)(AG * cc / d);
            sp[z * 12 + 7 + 2 * i] = (float)(PIK * PIK / d);
        }
    }
    // tabulated radial profiles of the species present (up to kPotMaxSp): cubic
    // pieces of vzatom evaluated in FP64 over [0.15 A, radius]
    std::vector<int> zlist, zslot(104, -1);
    for (int z = 1; z <= 103; ++z)
        if (used[z]) {
            zslot[z] = (int)zlist.size();
            zlist.push_back(z);
        }
    im.nsp = (zlist.size() <= (size_t)msl::kPotMaxSp && radius > 2 * im.tab_r0) ? (int)zlist.size() : 0;
    const size_t ntab = (size_t)std::max(im.nsp, 1) * msl::kPotTabN;
    if (im.tab_z != zlist || im.tab_radius != radius || im.tab_fp != fparams || im.tab.size() != ntab) {
        im.tab.assign(ntab, make_float4(0.f, 0.f, 0.f, 0.f));
        if (im.nsp) msl::potential_tables(fparams, zlist.data(), im.nsp, im.tab_r0, radius, im.tab.data());
        im.tab_z = zlist;
        im.tab_radius = radius;
        im.tab_fp = fparams;
    }
    auto up16 = [](size_t x) { return ((x + 15) / 16) * 16; };
    im.o_off = 0;
    im.o_ic = up16(sizeof(int) * (nslice + 1));
    im.o_jc = up16(im.o_ic + sizeof(int) * nk);
    im.o_fx = up16(im.o_jc + sizeof(int) * nk);
    im.o_fy = up16(im.o_fx + sizeof(float) * nk);
    im.o_z = up16(im.o_fy + sizeof(float) * nk);
    im.o_sp = up16(im.o_z + sizeof(int) * nk);
    im.o_xf = up16(im.o_sp + sizeof(float) * sp.size());
    im.o_yf = up16(im.o_xf + sizeof(float) * nk);
    im.o_tab = up16(im.o_yf + sizeof(float) * nk);
    im.o_zs = im.o_tab + sizeof(float4) * im.tab.size();
    im.h.assign(im.o_zs + sizeof(int) * zslot.size(), 0);
    unsigned char *h = im.h.data();
    int *ics = (int *)(h + im.o_ic), *jcs = (int *)(h + im.o_jc), *zs = (int *)(h + im.o_z);
    float *fxs = (float *)(h + im.o_fx), *fys = (float *)(h + im.o_fy);
    float *xf = (float *)(h + im.o_xf), *yf = (float *)(h + im.o_yf);
    const double dxp = g->ax / g->nx, dyp = g->by / g->ny;
    std::vector<int> fill(count.begin(), count.end() - 1);
    for (int i = 0; i < at->natom; ++i) {
        if (kz[i] < 0) continue;
        const int p = fill[kz[i]]++;
        const double xw = at->x[i] - g->ax * std::floor(at->x[i] / g->ax);
        const double yw = at->y[i] - g->by * std::floor(at->y[i] / g->by);
        // nearest pixel and the FP64 residue (the same expression as |x - ix dxp|
        // at that pixel); the pixel index is then wrapped into the grid
        const double ci = std::floor(xw / dxp + 0.5), cj = std::floor(yw / dyp + 0.5);
        fxs[p] = (float)(xw - ci * dxp);
        fys[p] = (float)(yw - cj * dyp);
        ics[p] = (int)ci % g->nx;
        jcs[p] = (int)cj % g->ny;
        zs[p] = at->Z[i];
        xf[p] = (float)xw;
        yf[p] = (float)yw;
    }
    memcpy(h + im.o_off, count.data(), sizeof(int) * (nslice + 1));
    memcpy(h + im.o_sp, sp.data(), sizeof(float) * sp.size());
    memcpy(h + im.o_tab, im.tab.data(), sizeof(float4) * im.tab.size());
    memcpy(h + im.o_zs, zslot.data(), sizeof(int) * zslot.size());
    return MSL_OK;
}

// Device half: launch the gather on the upload image at `d` (device memory).
int potential_launch(msl_ctx *c, const PotImage &im, const unsigned char *d, const msl_grid *g, int nslice,
                     double radius, float *vd) {
    msl::PotArgs a;
    a.ic = (const int *)(d + im.o_ic);
    a.jc = (const int *)(d + im.o_jc);
    a.fx = (const float *)(d + im.o_fx);
    a.fy = (const float *)(d + im.o_fy);
    a.xf = (const float *)(d + im.o_xf);
    a.yf = (const float *)(d + im.o_yf);
    a.Z = (const int *)(d + im.o_z);
    a.off = (const int *)(d + im.o_off);
    a.nslice = nslice;
    a.nx = g->nx;
    a.ny = g->ny;
    a.ax = g->ax;
    a.by = g->by;
    a.dxp = g->ax / g->nx;
    a.dyp = g->by / g->ny;
    a.dxpf = (float)a.dxp;
    a.dypf = (float)a.dyp;
    a.rad2 = (float)(radius * radius);
    a.sp = (const float *)(d + im.o_sp);
    a.v = vd;
    a.tab = (const float4 *)(d + im.o_tab);
    a.zslot = (const int *)(d + im.o_zs);
    a.nsp = im.nsp;
    a.tab_r0 = (float)im.tab_r0;
    a.tab_inv_h = (float)(msl::kPotTabN / (radius - im.tab_r0));
    a.tab_off = (float)(-im.tab_r0 * msl::kPotTabN / (radius - im.tab_r0));
    LAUNCH_TRY(c, timed(c, MSL_PROF_POTENTIAL, [&] { return msl::launch_potential(a, c->stream, &c->launches); }));
    return MSL_OK;
}

}  // namespace

namespace {

// t = exp(i sigma V) elementwise, then the band limit: forward transform, 2/3
// mask, inverse transform (mulslice.cpp:414-421, :515-522), on the context's
// stream; st holds the identity propagator tables of the grid.
int transmission_enqueue(msl_ctx *c, const msl_grid *g, const msl_optics *o, const float *vd, int nlayer,
                         float2 *td, const SliceTables &st, float2 *twr, float2 *twc) {
    const size_t n2 = (size_t)g->nx * g->ny;
    const double phase_scale = msl_sigma(o->kev) / 1000.0;  // rad per V*A
    LAUNCH_TRY(c, timed(c, MSL_PROF_OTHER, [&] {
                   return msl::launch_transmission_phase(vd, phase_scale, n2 * nlayer, td, c->nsm, c->stream,
                                                         &c->launches);
               }));
    RowArgs r = row_args(g, twr, nullptr, td, nlayer, msl::ROW_LOAD | msl::ROW_FWD, c->dflag);
    LAUNCH_TRY(c, timed(c, MSL_PROF_ROW, [&] { return msl::launch_row_pass(g->ny, r, c->stream, c->nsm, &c->launches); }));
    ColArgs ca = col_args(g, st, twc, 0, td, nlayer,
                          msl::COL_LOAD | msl::COL_FWD | msl::COL_PROP | msl::COL_INV | msl::COL_STORE, c->dflag);
    LAUNCH_TRY(c, timed(c, MSL_PROF_COL, [&] { return msl::launch_col_pass(g->nx, ca, c->stream, c->nsm, &c->launches); }));
    r = row_args(g, twr, nullptr, td, nlayer, msl::ROW_LOAD | msl::ROW_INV, c->dflag);
    LAUNCH_TRY(c, timed(c, MSL_PROF_ROW, [&] { return msl::launch_row_pass(g->ny, r, c->stream, c->nsm, &c->launches); }));
    return MSL_OK;
}

}  // namespace

namespace {

// Transmission functions of frozen-phonon configurations, built on the
// context's stream: each configuration's atoms are displaced
// (msl_phonon_displacements), binned and uploaded through one of two pinned
// buffers, its potential gathered and turned into band-limited transmission
// functions; the host work of the next configuration runs while the GPU builds
// the current one.  Nothing here synchronizes with the stream or checks the
// kernel error flag: the caller does both after its slice loop.
struct PhononBuilder {
    msl_ctx *c;
    const msl_atoms *at;
    const double *fparams;
    const msl_grid *g;
    const msl_optics *o;
    int nslice, nconfig;
    double radius, sigma;
    uint64_t seed;
    SliceTables st;
    float2 *twr = nullptr, *twc = nullptr;
    DevBuf tabs, atoms, pot;
    PotImage im[2];
    int prepared[2] = {-1, -1};
    unsigned char *pin[2] = {nullptr, nullptr};
    size_t pin_cap = 0;
    cudaEvent_t ev[2] = {nullptr, nullptr};
    std::vector<double> x, y, z, d;
    msl_atoms jat;

    PhononBuilder(msl_ctx *c_, const msl_atoms *at_, const double *fp, const msl_grid *g_, int nslice_,
                  double radius_, const msl_optics *o_, int nconfig_, double sigma_, uint64_t seed_)
        : c(c_), at(at_), fparams(fp), g(g_), o(o_), nslice(nslice_), nconfig(nconfig_), radius(radius_),
          sigma(sigma_), seed(seed_) {
        tabs.mb = atoms.mb = pot.mb = &c->mem;
    }
    ~PhononBuilder() {
        for (int i = 0; i < 2; ++i) {
            if (ev[i]) {
                cudaEventSynchronize(ev[i]);
                cudaEventDestroy(ev[i]);
            }
            if (pin[i]) cudaFreeHost(pin[i]);
        }
    }
    int init() {
        const int na = at->natom;
        x.resize(na);
        y.resize(na);
        z.resize(na);
        d.resize(3 * (size_t)na);
        jat = *at;
        jat.x = x.data();
        jat.y = y.data();
        jat.z = z.data();
        int rc;
        if ((rc = build_slice_tables(c, g, o, 1, nullptr, st, &tabs))) return rc;
        twr = twiddles(c, g->ny);
        twc = twiddles(c, g->nx);
        if (!twr || !twc) return fail(c, MSL_E_NOMEM, "twiddle table allocation failed");
        CUDA_TRY(c, pot.ensure(sizeof(float) * (size_t)nslice * g->nx * g->ny));
        for (int i = 0; i < 2; ++i) CUDA_TRY(c, cudaEventCreateWithFlags(&ev[i], cudaEventDisableTiming));
        return prepare(0);
    }
    int prepare(int cfg) {
        msl_phonon_displacements(seed, cfg, at->natom, sigma, d.data());
        for (int i = 0; i < at->natom; ++i) {
            x[i] = at->x[i] + d[3 * i];
            y[i] = at->y[i] + d[3 * i + 1];
            z[i] = at->z[i] + d[3 * i + 2];
        }
        const int rc = potential_prepare(c, &jat, fparams, g, nslice, radius, im[cfg & 1]);
        if (rc) return rc;
        prepared[cfg & 1] = cfg;
        return MSL_OK;
    }
    // Enqueue configuration cfg's transmission functions into t (device), then
    // prepare configuration cfg + 1 on the host.
    int build(int cfg, float2 *t) {
        int rc;
        const int sl = cfg & 1;
        if (prepared[sl] != cfg && (rc = prepare(cfg))) return rc;
        const PotImage &m = im[sl];
        const size_t bytes = m.h.size();
        if (bytes > pin_cap) {  // (re)allocate both pinned buffers with headroom
            for (int i = 0; i < 2; ++i) {
                CUDA_TRY(c, cudaEventSynchronize(ev[i]));
                if (pin[i]) cudaFreeHost(pin[i]);
                pin[i] = nullptr;
            }
            pin_cap = bytes + bytes / 4;
            for (int i = 0; i < 2; ++i) CUDA_TRY(c, cudaHostAlloc((void **)&pin[i], pin_cap, cudaHostAllocDefault));
        }
        if (bytes > atoms.cap) {  // growth frees the old buffer: let the stream drain first
            CUDA_TRY(c, cudaStreamSynchronize(c->stream));
            CUDA_TRY(c, atoms.ensure(bytes + bytes / 4));
        }
        CUDA_TRY(c, cudaEventSynchronize(ev[sl]));  // the upload two configurations back has read pin[sl]
        memcpy(pin[sl], m.h.data(), bytes);
        CUDA_TRY(c, cudaMemcpyAsync(atoms.p, pin[sl], bytes, cudaMemcpyHostToDevice, c->stream));
        CUDA_TRY(c, cudaEventRecord(ev[sl], c->stream));
        if ((rc = potential_launch(c, m, (const unsigned char *)atoms.p, g, nslice, radius, (float *)pot.p))) return rc;
        if ((rc = transmission_enqueue(c, g, o, (const float *)pot.p, nslice, t, st, twr, twc))) return rc;
        if (cfg + 1 < nconfig && (rc = prepare(cfg + 1))) return rc;
        return MSL_OK;
    }
};

}  // namespace

int msl_frozen_phonon(msl_ctx *c, const msl_atoms *at, const double *fparams, const msl_grid *g,
                      int nslice, double radius, const msl_optics *o, const msl_lens *lens, int nconfig,
                      double sigma, uint64_t seed, double *image, double *exit_intensity) {
    if (!c) return MSL_E_ARG;
    int rc = check_grid(c, g);
    if (rc) return rc;
    if ((rc = check_optics(c, o))) return rc;
    if ((rc = check_lens(c, lens))) return rc;
    if (!at || nconfig < 1 || !(sigma >= 0) || !is_fin(sigma) || nslice < 1)
        return fail(c, MSL_E_ARG, "atoms required, nconfig >= 1, sigma >= 0, nslice >= 1");
    if (!image && !exit_intensity) return fail(c, MSL_E_ARG, "nothing to compute: image and exit_intensity null");
    CUDA_TRY(c, cudaSetDevice(c->device));
    const int nx = g->nx, ny = g->ny;
    const size_t n2 = (size_t)nx * ny;
    // device buffers: potential (one configuration), transmissions of a batch of
    // configurations, their waves, accumulators.  The configurations of a batch
    // run through one slice loop, each with its own transmission functions
    // (per-image row pointers), and are imaged and accumulated in order, so the
    // sums equal the one-configuration-at-a-time loop bit for bit.
    const size_t slab = sizeof(float2) * n2 * nslice;  // one configuration's transmissions
    size_t budget = (size_t)16 << 30;
    if (c->mem.limit && c->mem.limit / 2 < budget) budget = c->mem.limit / 2;
    const int B = (int)std::max<size_t>(1, std::min<size_t>((size_t)nconfig, budget / (slab + sizeof(float2) * n2)));
    DevBuf tbuf, pbuf;
    tbuf.mb = pbuf.mb = &c->mem;
    CUDA_TRY(c, tbuf.ensure(slab * B));
    CUDA_TRY(c, pbuf.ensure(sizeof(float2 *) * (size_t)nslice * B));
    CUDA_TRY(c, c->acc.ensure(2 * sizeof(double) * n2));
    double *img_d = (double *)c->acc.p, *exit_d = img_d + n2;
    CUDA_TRY(c, cudaMemsetAsync(img_d, 0, 2 * sizeof(double) * n2, c->stream));
    CUDA_TRY(c, c->wave.ensure(sizeof(float2) * n2 * B));
    float2 *w = (float2 *)c->wave.p;
    float2 *tall = (float2 *)tbuf.p;
    const float2 **ptab = (const float2 **)pbuf.p;
    std::vector<const float2 *> hptab((size_t)nslice * B);
    std::vector<double> dz(nslice, at->cz / nslice);
    std::vector<int> seq(nslice);
    for (int s = 0; s < nslice; ++s) seq[s] = s;
    PhononBuilder pb(c, at, fparams, g, nslice, radius, o, nconfig, sigma, seed);
    int out = pb.init();
    if (out == MSL_OK) out = err_reset(c);
    for (int cfg0 = 0; cfg0 < nconfig && out == MSL_OK; cfg0 += B) {
        const int nb = std::min(B, nconfig - cfg0);
        for (int b = 0; b < nb && out == MSL_OK; ++b) {
            if ((out = pb.build(cfg0 + b, tall + n2 * nslice * b))) break;
            for (int s = 0; s < nslice; ++s) hptab[(size_t)s * nb + b] = tall + n2 * nslice * b + n2 * s;
        }
        if (out != MSL_OK) break;
        if (cudaMemcpyAsync(ptab, hptab.data(), sizeof(float2 *) * (size_t)nslice * nb, cudaMemcpyHostToDevice,
                            c->stream) != cudaSuccess) {
            out = fail(c, MSL_E_CUDA, "frozen phonon: transmission table upload failed");
            break;
        }
        if ((out = ctem_core(c, g, o, tall, nslice, dz.data(), seq.data(), nslice, lens, w, nb, true,
                             1.0 / nconfig, img_d, exit_intensity ? exit_d : nullptr, false, ptab)))
            break;
        cudaError_t e = cudaStreamSynchronize(c->stream);  // also: hptab is free for the next batch
        if (e != cudaSuccess) {
            out = fail(c, MSL_E_CUDA, std::string("frozen phonon: ") + cudaGetErrorString(e));
            break;
        }
        collect_profile(c);
        if ((out = err_check(c))) break;
    }
    if (out == MSL_OK) {
        if (image) {
            cudaError_t e = cudaMemcpyAsync(image, img_d, sizeof(double) * n2, cudaMemcpyDefault, c->stream);
            if (e != cudaSuccess) out = fail(c, MSL_E_CUDA, "copy of the image failed");
        }
        if (out == MSL_OK && exit_intensity) {
            cudaError_t e = cudaMemcpyAsync(exit_intensity, exit_d, sizeof(double) * n2, cudaMemcpyDefault, c->stream);
            if (e != cudaSuccess) out = fail(c, MSL_E_CUDA, "copy of the exit intensity failed");
        }
        cudaStreamSynchronize(c->stream);
    }
    cudaStreamSynchronize(c->stream);
    tbuf.release();
    pbuf.release();
    return out;
}


namespace {

// One grid shape of an uneven batch: its jobs (by decreasing slice count) and
// where its buffers sit in the call's arenas.
struct JobGroup {
    int nx = 0, ny = 0;
    std::vector<int> ids;
    size_t wave_off = 0, tab_off = 0, ptab_off = 0, stage_off = 0, apchi_off = 0, exy_off = 0;
    size_t kbytes = 0, nprop = 0;
    std::vector<std::vector<size_t>> layer_prop;  // per job, per layer: row of its propagator table
    float2 *twr = nullptr, *twc = nullptr;
};

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

cudaStream_t group_stream(msl_ctx *c, size_t i) {
    while (c->side_streams.size() <= i) {
        cudaStream_t s = nullptr;
        if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) return nullptr;
        c->side_streams.push_back(s);
    }
    return c->side_streams[i];
}

// Run the groups of an uneven batch: every host table first (one upload per
// arena), then each group's probe formation and lockstep slice loop on its
// own stream (the context stream when profiling), then the exit waves out.
int run_job_groups(msl_ctx *c, const msl_job *jobs, std::vector<JobGroup> &groups, double bandlimit) {
    size_t wave_bytes = 0, tab_bytes = 0, ptab_bytes = 0, stage_bytes = 0, apchi_bytes = 0, exy_bytes = 0;
    for (JobGroup &g : groups) {
        const size_t n2 = (size_t)g.nx * g.ny, nb = g.ids.size();
        const int S = jobs[g.ids[0]].nslice;
        g.twr = twiddles(c, g.ny);
        g.twc = twiddles(c, g.nx);
        if (!g.twr || !g.twc) return fail(c, MSL_E_NOMEM, "twiddle table allocation failed");
        // one propagator table per distinct slice thickness of a job (layers
        // of equal dz share it; the tables depend on nothing else)
        g.layer_prop.assign(nb, {});
        g.nprop = 0;
        bool probes = false;
        for (size_t b = 0; b < nb; ++b) {
            const msl_job &jb = jobs[g.ids[b]];
            std::map<uint64_t, size_t> seen;  // keyed by the bits of dz
            g.layer_prop[b].resize(jb.ntrans);
            for (int l = 0; l < jb.ntrans; ++l) {
                uint64_t key;
                memcpy(&key, &jb.dz[l], sizeof(key));
                auto it = seen.find(key);
                if (it == seen.end()) it = seen.emplace(key, g.nprop++).first;
                g.layer_prop[b][l] = it->second;
            }
            if (jb.illumination == MSL_PROBE) probes = true;
        }
        g.kbytes = sizeof(float) * (g.nx + g.ny) * nb;
        g.wave_off = wave_bytes;
        wave_bytes = align256(wave_bytes + sizeof(float2) * n2 * nb);
        g.tab_off = tab_bytes;
        tab_bytes = align256(tab_bytes + g.kbytes + sizeof(float2) * (g.nx + g.ny) * g.nprop);
        g.ptab_off = ptab_bytes;
        ptab_bytes = align256(ptab_bytes + sizeof(void *) * ((size_t)2 * S * nb + nb) + sizeof(float) * nb);
        g.stage_off = stage_bytes;
        for (size_t b = 0; b < nb; ++b)
            if (!on_device(jobs[g.ids[b]].trans))
                stage_bytes = align256(stage_bytes + sizeof(float2) * n2 * jobs[g.ids[b]].ntrans);
        g.apchi_off = apchi_bytes;
        g.exy_off = exy_bytes;
        if (probes) {
            apchi_bytes = align256(apchi_bytes + sizeof(float2) * n2 + n2);
            exy_bytes = align256(exy_bytes + sizeof(float2) * (g.nx + g.ny));
        }
    }
    size_t fxy_len = 0;
    for (JobGroup &g : groups)
        for (int j : g.ids)
            if (jobs[j].illumination == MSL_PROBE) fxy_len += (size_t)g.nx + g.ny + 2;
    // a column of ones (the plane wave's ky = 0 column) after the tables
    const size_t ones_off = tab_bytes;
    tab_bytes = align256(tab_bytes + sizeof(float2) * 2048);
    CUDA_TRY(c, c->wave.ensure(wave_bytes));
    CUDA_TRY(c, c->tabs.ensure(tab_bytes));
    CUDA_TRY(c, c->jobtab.ensure(ptab_bytes));
    CUDA_TRY(c, c->trans_stage.ensure(stage_bytes));
    CUDA_TRY(c, c->apchi.ensure(apchi_bytes));
    CUDA_TRY(c, c->exy.ensure(exy_bytes));
    CUDA_TRY(c, c->fxy.ensure(sizeof(double) * fxy_len));
    unsigned char *dtab = (unsigned char *)c->tabs.p, *dptab = (unsigned char *)c->jobtab.p;
    std::vector<unsigned char> htab(tab_bytes), hptab(ptab_bytes);
    std::vector<double> hk(fxy_len);
    for (int i = 0; i < 2048; ++i) ((float2 *)(htab.data() + ones_off))[i] = make_float2(1.f, 0.f);
    size_t fo = 0;
    for (JobGroup &g : groups) {
        const int nx = g.nx, ny = g.ny, nb = (int)g.ids.size(), S = jobs[g.ids[0]].nslice;
        const size_t n2 = (size_t)nx * ny;
        // transmission stacks on the device (staged when on the host)
        std::vector<const float2 *> tdev(nb);
        size_t so = g.stage_off;
        for (int b = 0; b < nb; ++b) {
            const msl_job &jb = jobs[g.ids[b]];
            if (on_device(jb.trans)) {
                tdev[b] = (const float2 *)jb.trans;
            } else {
                const size_t bytes = sizeof(float2) * n2 * jb.ntrans;
                float2 *dst = (float2 *)((unsigned char *)c->trans_stage.p + so);
                CUDA_TRY(c, cudaMemcpyAsync(dst, jb.trans, bytes, cudaMemcpyHostToDevice, c->stream));
                tdev[b] = dst;
                so = align256(so + bytes);
            }
        }
        // tables: [kx2 ky2] floats per job, then [px py] per distinct thickness
        float *hk2 = (float *)(htab.data() + g.tab_off);
        float2 *hprop = (float2 *)(htab.data() + g.tab_off + g.kbytes);
        std::vector<float> k2max(nb);
        for (int b = 0; b < nb; ++b) {
            const msl_job &jb = jobs[g.ids[b]];
            std::vector<float> kx, kx2, ky, ky2;
            freqn_f32(nx, jb.grid.ax, kx, kx2);
            freqn_f32(ny, jb.grid.by, ky, ky2);
            memcpy(hk2 + (size_t)b * (nx + ny), kx2.data(), sizeof(float) * nx);
            memcpy(hk2 + (size_t)b * (nx + ny) + nx, ky2.data(), sizeof(float) * ny);
            k2max[b] = k2max_f32(nx, ny, jb.grid.ax, jb.grid.by, bandlimit);
            msl_optics o = {jb.kev, bandlimit, 0.0, 0.0, 0};
            std::vector<char> done(g.nprop, 0);
            for (int l = 0; l < jb.ntrans; ++l) {
                const size_t row = g.layer_prop[b][l];
                if (done[row]) continue;
                done[row] = 1;
                float2 *pt = hprop + row * (nx + ny);
                prop_tables(nx, ny, jb.grid.ax, jb.grid.by, &o, jb.dz[l], kx, kx2, ky, ky2, pt, pt + nx);
            }
        }
        // pointer tables: trans[S][nb], prop[S][nb], k2[nb], then k2max[nb]
        const float *dk = (const float *)(dtab + g.tab_off);
        const float2 *dp = (const float2 *)(dtab + g.tab_off + g.kbytes);
        const void **pt = (const void **)(hptab.data() + g.ptab_off);
        for (int s = 0; s < S; ++s)
            for (int b = 0; b < nb; ++b) {
                const msl_job &jb = jobs[g.ids[b]];
                const int l = s < jb.nslice ? jb.layer_seq[s] : 0;
                pt[(size_t)s * nb + b] = tdev[b] + (size_t)l * n2;
                pt[(size_t)(S + s) * nb + b] = dp + g.layer_prop[b][l] * (nx + ny);
            }
        for (int b = 0; b < nb; ++b) pt[(size_t)2 * S * nb + b] = dk + (size_t)b * (nx + ny);
        memcpy(pt + (size_t)2 * S * nb + nb, k2max.data(), sizeof(float) * nb);
        // probe k-vectors and positions
        for (int b = 0; b < nb; ++b) {
            const msl_job &jb = jobs[g.ids[b]];
            if (jb.illumination != MSL_PROBE) continue;
            double *h = hk.data() + fo;
            for (int i = 0; i < nx; ++i) h[i] = (double)(i < nx / 2 ? i : i - nx) / jb.grid.ax;
            for (int i = 0; i < ny; ++i) h[nx + i] = (double)(i < ny / 2 ? i : i - ny) / jb.grid.by;
            h[nx + ny] = jb.probe_x / jb.grid.ax;
            h[nx + ny + 1] = jb.probe_y / jb.grid.by;
            fo += (size_t)nx + ny + 2;
        }
    }
    if (tab_bytes) CUDA_TRY(c, cudaMemcpyAsync(dtab, htab.data(), tab_bytes, cudaMemcpyHostToDevice, c->stream));
    if (ptab_bytes) CUDA_TRY(c, cudaMemcpyAsync(dptab, hptab.data(), ptab_bytes, cudaMemcpyHostToDevice, c->stream));
    if (fxy_len)
        CUDA_TRY(c, cudaMemcpyAsync(c->fxy.p, hk.data(), sizeof(double) * fxy_len, cudaMemcpyHostToDevice, c->stream));
    CUDA_TRY(c, cudaMemsetAsync(c->wave.p, 0, wave_bytes, c->stream));
    const bool concurrent = !c->prof && groups.size() > 1;
    cudaEvent_t fork = take_event(c);
    std::vector<cudaEvent_t> joins;
    CUDA_TRY(c, cudaEventRecord(fork, c->stream));
    const float2 *ones = (const float2 *)(dtab + ones_off);
    // on a failure after launches began, let every group stream drain before
    // returning (the next call reuses the buffers)
    auto drain = [&](int rc_) {
        if (concurrent)
            for (size_t gi = 0; gi < groups.size() && gi < c->side_streams.size(); ++gi)
                cudaStreamSynchronize(c->side_streams[gi]);
        cudaStreamSynchronize(c->stream);
        return rc_;
    };
    fo = 0;
    int lrc = [&]() -> int {
    for (size_t gi = 0; gi < groups.size(); ++gi) {
        JobGroup &g = groups[gi];
        const int nx = g.nx, ny = g.ny, nb = (int)g.ids.size(), S = jobs[g.ids[0]].nslice;
        const size_t n2 = (size_t)nx * ny;
        cudaStream_t st = c->stream;
        if (concurrent) {
            st = group_stream(c, gi);
            if (!st) return fail(c, MSL_E_CUDA, "stream creation failed");
            CUDA_TRY(c, cudaStreamWaitEvent(st, fork, 0));
        }
        float2 *w = (float2 *)((unsigned char *)c->wave.p + g.wave_off);
        const unsigned char *tp = dptab + g.ptab_off;
        const float2 *const *ttab = (const float2 *const *)tp;
        const float2 *const *ptabd = ttab + (size_t)S * nb;
        const float *const *ktab = (const float *const *)(ttab + (size_t)2 * S * nb);
        const float *dk2max = (const float *)(ktab + nb);
        // entrance waves in the column-inverse representation every job shares:
        // a plane wave is 1 in the ky = 0 column, a probe is ifft_x of its spectrum
        float2 *apchi = (float2 *)((unsigned char *)c->apchi.p + g.apchi_off);
        float2 *ex = (float2 *)((unsigned char *)c->exy.p + g.exy_off), *ey = ex + nx;
        for (int b = 0; b < nb; ++b) {
            const msl_job &jb = jobs[g.ids[b]];
            float2 *slot = w + (size_t)b * n2;
            if (jb.illumination == MSL_PLANE_WAVE) {
                CUDA_TRY(c, cudaMemcpy2DAsync(slot, sizeof(float2) * ny, ones, sizeof(float2),
                                              sizeof(float2), nx, cudaMemcpyDeviceToDevice, st));
                continue;
            }
            const double *kxd = (const double *)c->fxy.p + fo, *kyd = kxd + nx;
            fo += (size_t)nx + ny + 2;
            LAUNCH_TRY(c, timed(c, MSL_PROF_OTHER, [&] {
                           return msl::launch_probe_table(nx, ny, kxd, kyd, jb.probe.k_in * jb.probe.k_in,
                                                          jb.probe.k_out * jb.probe.k_out, msl_wavelength(jb.kev),
                                                          jb.probe.df, jb.probe.cs, 1.0 / ((double)nx * ny), apchi,
                                                          st, &c->launches);
                       }));
            LAUNCH_TRY(c, timed(c, MSL_PROF_OTHER, [&] {
                           return msl::launch_probe_shifts(nx, ny, 1, kyd + ny, ex, ey, st, &c->launches);
                       }));
            SliceTables none;
            none.k2max = 0.f;
            none.d_kx2 = none.d_ky2 = nullptr;
            none.d_prop = nullptr;
            ColArgs pa = col_args(&jb.grid, none, g.twc, 0, slot, 1, msl::COL_PROBE | msl::COL_INV | msl::COL_STORE,
                                  c->dflag);
            pa.apchi = apchi;
            pa.ex = ex;
            pa.ey = ey;
            LAUNCH_TRY(c, timed(c, MSL_PROF_COL, [&] { return msl::launch_col_pass(nx, pa, st, c->nsm, &c->launches); }));
        }
        // lockstep slice loop over the running prefix
        msl_grid gg = {nx, ny, 1.0, 1.0};
        SliceTables none;
        none.k2max = 0.f;
        none.d_kx2 = none.d_ky2 = nullptr;
        none.d_prop = nullptr;
        for (int s = 0; s < S; ++s) {
            int nact = 0;
            while (nact < nb && jobs[g.ids[nact]].nslice > s) ++nact;
            RowArgs r = row_args(&gg, g.twr, nullptr, w, nact,
                                 msl::ROW_LOAD | msl::ROW_INV | msl::ROW_TRANS | msl::ROW_FWD, c->dflag);
            r.trans_b = ttab + (size_t)s * nb;
            LAUNCH_TRY(c, timed(c, MSL_PROF_ROW, [&] { return msl::launch_row_pass(ny, r, st, c->nsm, &c->launches); }));
            ColArgs ca = col_args(&gg, none, g.twc, 0, w, nact,
                                  msl::COL_LOAD | msl::COL_FWD | msl::COL_PROP | msl::COL_INV | msl::COL_STORE, c->dflag);
            ca.prop_b = ptabd + (size_t)s * nb;
            ca.k2_b = ktab;
            ca.k2max_b = dk2max;
            LAUNCH_TRY(c, timed(c, MSL_PROF_COL, [&] { return msl::launch_col_pass(nx, ca, st, c->nsm, &c->launches); }));
        }
        RowArgs r = row_args(&gg, g.twr, nullptr, w, nb, msl::ROW_LOAD | msl::ROW_INV, c->dflag);
        LAUNCH_TRY(c, timed(c, MSL_PROF_ROW, [&] { return msl::launch_row_pass(ny, r, st, c->nsm, &c->launches); }));
        if (concurrent) {
            cudaEvent_t e = take_event(c);
            joins.push_back(e);
            CUDA_TRY(c, cudaEventRecord(e, st));
        }
    }
    return MSL_OK;
    }();
    if (lrc) return drain(lrc);
    for (cudaEvent_t e : joins) CUDA_TRY(c, cudaStreamWaitEvent(c->stream, e, 0));
    // exit waves out once every group's loop has been issued
    for (JobGroup &g : groups) {
        const size_t n2 = (size_t)g.nx * g.ny;
        const float2 *w = (const float2 *)((unsigned char *)c->wave.p + g.wave_off);
        for (size_t b = 0; b < g.ids.size(); ++b)
            CUDA_TRY(c, cudaMemcpyAsync(jobs[g.ids[b]].exit_wave, w + b * n2, sizeof(float2) * n2,
                                        cudaMemcpyDefault, c->stream));
    }
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    c->ev_free.push_back(fork);
    for (cudaEvent_t e : joins) c->ev_free.push_back(e);
    return MSL_OK;
}

}  // namespace

int msl_run_jobs(msl_ctx *c, const msl_job *jobs, int njobs, double bandlimit) {
    if (!c) return MSL_E_ARG;
    if (!jobs || njobs < 1) return fail(c, MSL_E_ARG, "jobs required");
    if (!(bandlimit > 0) || bandlimit > 1.0) return fail(c, MSL_E_ARG, "bandlimit must lie in (0, 1]");
    int rc;
    for (int j = 0; j < njobs; ++j) {
        const msl_job &jb = jobs[j];
        msl_optics o = {jb.kev, bandlimit, 0.0, 0.0, 0};
        if ((rc = check_grid(c, &jb.grid)) || (rc = check_optics(c, &o)) ||
            (rc = check_layers(c, jb.ntrans, jb.dz, jb.layer_seq, jb.nslice))) {
            c->err = "job " + std::to_string(j) + ": " + c->err;
            return rc;
        }
        if (!jb.trans || !jb.exit_wave) return fail(c, MSL_E_ARG, "job " + std::to_string(j) + ": trans/exit_wave null");
        if (jb.illumination != MSL_PLANE_WAVE && jb.illumination != MSL_PROBE)
            return fail(c, MSL_E_ARG, "job " + std::to_string(j) + ": unknown illumination");
        if (jb.illumination == MSL_PROBE &&
            (!(jb.probe.k_in >= 0) || !(jb.probe.k_out > jb.probe.k_in) || !is_fin(jb.probe.k_out) ||
             !is_fin(jb.probe.df) || !is_fin(jb.probe.cs) || !is_fin(jb.probe_x) || !is_fin(jb.probe_y)))
            return fail(c, MSL_E_ARG, "job " + std::to_string(j) + ": invalid probe");
    }
    CUDA_TRY(c, cudaSetDevice(c->device));
    if ((rc = err_reset(c))) return rc;
    // group by grid shape
    std::map<std::pair<int, int>, std::vector<int>> gmap;
    for (int j = 0; j < njobs; ++j) gmap[{jobs[j].grid.nx, jobs[j].grid.ny}].push_back(j);
    std::vector<JobGroup> groups;
    for (auto &kv : gmap) {
        JobGroup g;
        g.nx = kv.first.first;
        g.ny = kv.first.second;
        g.ids = kv.second;
        std::stable_sort(g.ids.begin(), g.ids.end(), [&](int x, int y) { return jobs[x].nslice > jobs[y].nslice; });
        groups.push_back(std::move(g));
    }
    // Without a memory cap every group's buffers coexist and the groups run
    // concurrently, one stream each; under a cap they run one after another
    // in the same buffers.
    if (c->mem.limit) {
        for (auto &g : groups) {
            std::vector<JobGroup> one(1, std::move(g));
            if ((rc = run_job_groups(c, jobs, one, bandlimit))) return rc;
        }
    } else if ((rc = run_job_groups(c, jobs, groups, bandlimit))) {
        return rc;
    }
    collect_profile(c);
    if (c->dflag && (rc = err_check(c))) return rc;
    return MSL_OK;
}


int msl_ctem_partial_coherence(msl_ctx *c, const msl_grid *g, const msl_optics *o, const float *trans,
                               int ntrans, const double *dz, const int *layer_seq, int nslice,
                               const msl_lens *lens, double acmin, double acmax, double *image,
                               int *n_angles) {
    if (!c) return MSL_E_ARG;
    int rc = check_grid(c, g);
    if (rc) return rc;
    if ((rc = check_optics(c, o))) return rc;
    if ((rc = check_layers(c, ntrans, dz, layer_seq, nslice))) return rc;
    if ((rc = check_lens(c, lens))) return rc;
    if (!trans || !image) return fail(c, MSL_E_ARG, "trans and image required");
    if (!(acmin >= 0) || !(acmax >= acmin) || !is_fin(acmax))
        return fail(c, MSL_E_ARG, "illumination angles must satisfy 0 <= acmin <= acmax");
    CUDA_TRY(c, cudaSetDevice(c->device));
    if ((rc = err_reset(c))) return rc;
    const int nx = g->nx, ny = g->ny;
    const size_t n2 = (size_t)nx * ny;
    // illumination angles in float as mulslice.cpp:550-570
    const float wavlen = (float)msl_wavelength(o->kev);
    const float ax = (float)g->ax, by = (float)g->by;
    const float rx = 1.0F / ax, ry = 1.0F / by;
    const float fac = (float)acmax;
    const int nacx = (int)((fac / (wavlen * rx)) + 1.5F), nacy = (int)((fac / (wavlen * ry)) + 1.5F);
    float q2max = fac / wavlen;
    q2max = q2max * q2max;
    float q2min = (float)acmin / wavlen;
    q2min = q2min * q2min;
    std::vector<float> q;
    for (int iqy = -nacy; iqy <= nacy; ++iqy) {
        const float qy = iqy * ry, qy2 = qy * qy;
        for (int iqx = -nacx; iqx <= nacx; ++iqx) {
            const float qx = iqx * rx, q2 = qx * qx + qy2;
            if (q2 <= q2max && q2 >= q2min) {
                q.push_back(qx);
                q.push_back(qy);
            }
        }
    }
    const int na = (int)(q.size() / 2);
    if (n_angles) *n_angles = na;
    if (na == 0) return fail(c, MSL_E_ARG, "no illumination angle inside [acmin, acmax]");
    const float2 *td;
    if ((rc = stage_in(c, (const float2 *)trans, sizeof(float2) * n2 * ntrans, c->trans_stage, &td))) return rc;
    // positions xo[i] = (float)(i * a) / (float)(n - 1) of freqn (slicelib.cpp:433-463), and the angles
    std::vector<float> hp(nx + ny + q.size());
    for (int i = 0; i < nx; ++i) hp[i] = ((float)(i * g->ax)) / ((float)(nx - 1));
    for (int i = 0; i < ny; ++i) hp[nx + i] = ((float)(i * g->by)) / ((float)(ny - 1));
    memcpy(hp.data() + nx + ny, q.data(), sizeof(float) * q.size());
    if ((rc = upload(c, c->fxy, hp.data(), sizeof(float) * hp.size()))) return rc;
    const float *dpos = (const float *)c->fxy.p;
    CUDA_TRY(c, c->wave.ensure(sizeof(float2) * n2 * na));
    float2 *w = (float2 *)c->wave.p;
    LAUNCH_TRY(c, timed(c, MSL_PROF_OTHER, [&] {
                   return msl::launch_tilt_waves(nx, ny, na, dpos, dpos + nx, dpos + nx + ny, w, c->stream,
                                                 &c->launches);
               }));
    const bool idev = on_device(image);
    CUDA_TRY(c, c->acc.ensure(sizeof(double) * n2));
    double *img_d = idev ? image : (double *)c->acc.p;
    CUDA_TRY(c, cudaMemsetAsync(img_d, 0, sizeof(double) * n2, c->stream));
    if ((rc = ctem_core(c, g, o, td, ntrans, dz, layer_seq, nslice, lens, w, na, false, 1.0 / na, img_d,
                        nullptr, false, nullptr)))
        return rc;
    if (!idev) CUDA_TRY(c, cudaMemcpyAsync(image, img_d, sizeof(double) * n2, cudaMemcpyDeviceToHost, c->stream));
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    collect_profile(c);
    if (c->dflag && (rc = err_check(c))) return rc;
    return MSL_OK;
}

int msl_check_wait_timeout(msl_ctx *c, uint32_t polls) {
    if (!c) return MSL_E_ARG;
    if (polls == 0 || polls > (1u << 20)) return fail(c, MSL_E_ARG, "polls must lie in [1, 2^20]");
    CUDA_TRY(c, cudaSetDevice(c->device));
    int rc;
    if ((rc = err_reset(c))) return rc;
    LAUNCH_TRY(c, msl::launch_wait_timeout(c->dflag, polls, c->stream, &c->launches));
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    int h = 0;
    CUDA_TRY(c, cudaMemcpy(&h, c->dflag, sizeof(int), cudaMemcpyDeviceToHost));
    CUDA_TRY(c, cudaMemsetAsync(c->dflag, 0, sizeof(int), c->stream));
    if (h != 1) return fail(c, MSL_E_CUDA, "the bounded wait did not report its timeout");
    return MSL_OK;
}

int msl_set_memory_limit(msl_ctx *c, size_t bytes) {
    if (!c) return MSL_E_ARG;
    c->mem.limit = bytes;
    return MSL_OK;
}

int msl_memory_in_use(msl_ctx *c, size_t *bytes) {
    if (!c || !bytes) return MSL_E_ARG;
    *bytes = c->mem.used;
    return MSL_OK;
}

int msl_autotune(msl_ctx *c, int side, int batch, int reps, int *row_family, int *col_family, double *ms) {
    if (!c) return MSL_E_ARG;
    if (!msl::plan_supported(side)) return fail(c, MSL_E_UNSUPPORTED, "side not supported");
    if (batch < 1 || reps < 1) return fail(c, MSL_E_ARG, "batch and reps must be >= 1");
    CUDA_TRY(c, cudaSetDevice(c->device));
    int rc = err_reset(c);
    if (rc) return rc;
    int rf = 0, cf = 0;
    if ((rc = tune_side(c, side, batch, reps, &rf, &cf, ms))) return rc;
    if (c->device >= 0 && c->device < 64) g_tuned[c->device].fetch_or(1u << side_bit(side));
    if (row_family) *row_family = rf;
    if (col_family) *col_family = cf;
    return MSL_OK;
}

int msl_set_schedule(msl_ctx *c, int side, int row_family, int col_family) {
    if (!c) return MSL_E_ARG;
    CUDA_TRY(c, cudaSetDevice(c->device));
    if (!msl::set_schedule(side, row_family, col_family))
        return fail(c, MSL_E_ARG, "unknown side or pass family (0 fast, 1 TMA, 2 register)");
    if (c->device >= 0 && c->device < 64) g_tuned[c->device].fetch_or(1u << side_bit(side));
    return MSL_OK;
}

int msl_get_schedule(msl_ctx *c, int side, int *row_family, int *col_family) {
    if (!c || !row_family || !col_family) return MSL_E_ARG;
    CUDA_TRY(c, cudaSetDevice(c->device));
    if (!msl::get_schedule(side, row_family, col_family)) return fail(c, MSL_E_ARG, "unknown side");
    return MSL_OK;
}

int msl_set_autotune(msl_ctx *c, int on) {
    if (!c) return MSL_E_ARG;
    c->autotune = on != 0;
    return MSL_OK;
}

int msl_set_probe_batch(msl_ctx *c, int batch) {
    if (!c || batch < 0) return fail(c, MSL_E_ARG, "probe batch must be >= 0");
    c->probe_batch = batch;
    return MSL_OK;
}

int msl_fparams_parse(const char *text, size_t len, double *tab) {
    if (!text || !tab) return MSL_E_ARG;
    std::string s(text, len);
    memset(tab, 0, sizeof(double) * 104 * 12);
    size_t pos = 0;
    int seen = 0;
    while ((pos = s.find("Z=", pos)) != std::string::npos) {
        int z = atoi(s.c_str() + pos + 2);
        size_t eol = s.find('\n', pos);
        if (eol == std::string::npos) return MSL_E_ARG;
        const char *p = s.c_str() + eol + 1;
        double v[12];
        for (int i = 0; i < 12; ++i) {
            char *end = nullptr;
            v[i] = strtod(p, &end);
            if (end == p) return MSL_E_ARG;
            p = end;
        }
        if (z < 1 || z > 103) return MSL_E_ARG;
        for (int i = 0; i < 12; ++i) tab[z * 12 + i] = v[i];
        ++seen;
        pos = (size_t)(p - s.c_str());
    }
    return seen == 103 ? MSL_OK : MSL_E_ARG;
}

int msl_coo_parse(const char *text, size_t len, msl_cell *cell, double *rec, int capacity) {
    if (!text || !cell) return MSL_E_ARG;
    // split into lines, strip "//" comments, keep non-blank ones
    std::vector<std::string> lines;
    size_t p = 0;
    while (p < len) {
        size_t e = p;
        while (e < len && text[e] != '\n') ++e;
        std::string ln(text + p, e - p);
        const size_t cm = ln.find("//");
        if (cm != std::string::npos) ln = ln.substr(0, cm);
        for (char &ch : ln)
            if (ch == ',' || ch == '\r' || ch == '\t') ch = ch == ',' ? '.' : ' ';
        if (ln.find_first_not_of(' ') != std::string::npos) lines.push_back(ln);
        p = e + 1;
    }
    auto numbers = [](const std::string &ln, double *v, int maxn) {
        const char *q = ln.c_str();
        int n = 0;
        while (n < maxn) {
            char *end = nullptr;
            const double x = strtod(q, &end);
            if (end == q) break;
            v[n++] = x;
            q = end;
        }
        while (*q == ' ') ++q;
        return *q ? -1 : n;  // trailing junk: not a numeric line
    };
    size_t li = 0;
    double h[8];
    if (lines.empty()) return MSL_E_ARG;
    if (numbers(lines[0], h, 8) != 7) li = 1;  // a title line
    if (li >= lines.size() || numbers(lines[li], h, 8) != 7) return MSL_E_ARG;
    cell->a = h[0];
    cell->b = h[1];
    cell->c = h[2];
    cell->alpha = h[3];
    cell->beta = h[4];
    cell->gamma = h[5];
    if (!(h[6] >= 0) || h[6] > 2e9) return MSL_E_ARG;
    const int natom = (int)h[6];
    cell->natom = natom;
    if (!rec) return MSL_OK;
    if (capacity < natom) return MSL_E_ARG;
    if (lines.size() < li + 1 + (size_t)natom) return MSL_E_ARG;
    for (int k = 0; k < natom; ++k) {
        double v[8] = {0, 0, 0, 0, 0, 0, 1, 0};
        const int n = numbers(lines[li + 1 + k], v, 7);
        if (n < 4) return MSL_E_ARG;
        if (n < 5) v[4] = 0;
        if (n < 6) v[5] = 0;
        if (n < 7) v[6] = 1;
        for (int d = 0; d < 3; ++d) v[d] -= std::floor(v[d]);
        for (int d = 0; d < 7; ++d) rec[(size_t)k * 7 + d] = v[d];
    }
    return MSL_OK;
}

int msl_potential_build(msl_ctx *c, const msl_atoms *at, const double *fparams, const msl_grid *g,
                        int nslice, double radius, float *v_out) {
    if (!c) return MSL_E_ARG;
    int rc = check_grid(c, g);
    if (rc) return rc;
    if (!v_out) return fail(c, MSL_E_ARG, "null argument");
    PotImage im;
    if ((rc = potential_prepare(c, at, fparams, g, nslice, radius, im))) return rc;
    CUDA_TRY(c, cudaSetDevice(c->device));
    if ((rc = upload(c, c->atoms, im.h.data(), im.h.size()))) return rc;
    const size_t vbytes = sizeof(float) * (size_t)nslice * g->nx * g->ny;
    float *vd;
    const bool vdev = on_device(v_out);
    if (vdev) {
        vd = v_out;
    } else {
        CUDA_TRY(c, c->pot.ensure(vbytes));
        vd = (float *)c->pot.p;
    }
    if ((rc = potential_launch(c, im, (const unsigned char *)c->atoms.p, g, nslice, radius, vd))) return rc;
    if (!vdev) CUDA_TRY(c, cudaMemcpyAsync(v_out, vd, vbytes, cudaMemcpyDeviceToHost, c->stream));
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    collect_profile(c);
    return MSL_OK;
}

int msl_transmission_build(msl_ctx *c, const msl_grid *g, const msl_optics *o, const float *v,
                           int nlayer, float *t_out) {
    if (!c) return MSL_E_ARG;
    int rc = check_grid(c, g);
    if (rc) return rc;
    if ((rc = check_optics(c, o))) return rc;
    if (!v || !t_out || nlayer < 1) return fail(c, MSL_E_ARG, "null argument or nlayer < 1");
    CUDA_TRY(c, cudaSetDevice(c->device));
    if ((rc = err_reset(c))) return rc;
    const int nx = g->nx, ny = g->ny;
    const size_t n2 = (size_t)nx * ny;
    const float *vd;
    if ((rc = stage_in(c, v, sizeof(float) * n2 * nlayer, c->in_stage, &vd))) return rc;
    float2 *td;
    const bool tdev = on_device(t_out);
    if (tdev) {
        td = (float2 *)t_out;
    } else {
        CUDA_TRY(c, c->wave.ensure(sizeof(float2) * n2 * nlayer));
        td = (float2 *)c->wave.p;
    }
    SliceTables st;
    if ((rc = build_slice_tables(c, g, o, 1, nullptr, st))) return rc;
    float2 *twr = twiddles(c, ny), *twc = twiddles(c, nx);
    if (!twr || !twc) return fail(c, MSL_E_NOMEM, "twiddle table allocation failed");
    if ((rc = transmission_enqueue(c, g, o, vd, nlayer, td, st, twr, twc))) return rc;
    if (!tdev)
        CUDA_TRY(c, cudaMemcpyAsync(t_out, td, sizeof(float2) * n2 * nlayer, cudaMemcpyDeviceToHost,
                                    c->stream));
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    collect_profile(c);
    if (c->dflag && (rc = err_check(c))) return rc;
    return MSL_OK;
}

int msl_fft2d(msl_ctx *c, const msl_grid *g, float *psi, int batch, int dir) {
    if (!c) return MSL_E_ARG;
    int rc = check_grid(c, g);
    if (rc) return rc;
    if (!psi || batch < 1 || (dir != 1 && dir != -1))
        return fail(c, MSL_E_ARG, "psi must be non-null, batch >= 1, dir = +1 or -1");
    CUDA_TRY(c, cudaSetDevice(c->device));
    if ((rc = err_reset(c))) return rc;
    const int nx = g->nx, ny = g->ny;
    const size_t bytes = sizeof(float2) * (size_t)nx * ny * batch;
    const bool dev = on_device(psi);
    float2 *w;
    if (dev) {
        w = (float2 *)psi;
    } else {
        CUDA_TRY(c, c->wave.ensure(bytes));
        w = (float2 *)c->wave.p;
        CUDA_TRY(c, cudaMemcpyAsync(w, psi, bytes, cudaMemcpyHostToDevice, c->stream));
    }
    float2 *twr = twiddles(c, ny), *twc = twiddles(c, nx);
    if (!twr || !twc) return fail(c, MSL_E_NOMEM, "twiddle table allocation failed");
    SliceTables st;
    memset(&st.k2max, 0, sizeof(st.k2max));
    st.d_kx2 = nullptr;
    st.d_ky2 = nullptr;
    st.d_prop = nullptr;
    if (dir > 0) {
        RowArgs r = row_args(g, twr, nullptr, w, batch, msl::ROW_LOAD | msl::ROW_FWD, c->dflag);
        LAUNCH_TRY(c, timed(c, MSL_PROF_ROW, [&] { return msl::launch_row_pass(ny, r, c->stream, c->nsm, &c->launches); }));
        ColArgs ca = col_args(g, st, twc, 0, w, batch, msl::COL_LOAD | msl::COL_FWD | msl::COL_STORE, c->dflag);
        LAUNCH_TRY(c, timed(c, MSL_PROF_COL, [&] { return msl::launch_col_pass(nx, ca, c->stream, c->nsm, &c->launches); }));
    } else {
        ColArgs ca = col_args(g, st, twc, 0, w, batch, msl::COL_LOAD | msl::COL_INV | msl::COL_STORE, c->dflag);
        LAUNCH_TRY(c, timed(c, MSL_PROF_COL, [&] { return msl::launch_col_pass(nx, ca, c->stream, c->nsm, &c->launches); }));
        RowArgs r = row_args(g, twr, nullptr, w, batch, msl::ROW_LOAD | msl::ROW_INV, c->dflag);
        r.scale = 1.0f / ((float)nx * (float)ny);
        LAUNCH_TRY(c, timed(c, MSL_PROF_ROW, [&] { return msl::launch_row_pass(ny, r, c->stream, c->nsm, &c->launches); }));
    }
    if (!dev) CUDA_TRY(c, cudaMemcpyAsync(psi, w, bytes, cudaMemcpyDeviceToHost, c->stream));
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    collect_profile(c);
    if (c->dflag && (rc = err_check(c))) return rc;
    return MSL_OK;
}

int msl_multislice(msl_ctx *c, const msl_grid *g, const msl_optics *o, const float *trans,
                   int ntrans, const double *dz, const int *layer_seq, int nslice, float *psi,
                   int batch, int plane_wave) {
    if (!c) return MSL_E_ARG;
    int rc = check_grid(c, g);
    if (rc) return rc;
    if ((rc = check_optics(c, o))) return rc;
    if ((rc = check_layers(c, ntrans, dz, layer_seq, nslice))) return rc;
    if (!trans || !psi || batch < 1) return fail(c, MSL_E_ARG, "trans/psi null or batch < 1");
    CUDA_TRY(c, cudaSetDevice(c->device));
    if ((rc = maybe_tune(c, g->nx)) || (g->ny != g->nx && (rc = maybe_tune(c, g->ny)))) return rc;
    if ((rc = err_reset(c))) return rc;
    const int nx = g->nx, ny = g->ny;
    const size_t n2 = (size_t)nx * ny;
    const float2 *td;
    if ((rc = stage_in(c, (const float2 *)trans, sizeof(float2) * n2 * ntrans, c->trans_stage, &td)))
        return rc;
    const bool dev = on_device(psi);
    const size_t wbytes = sizeof(float2) * n2 * batch;
    float2 *w;
    if (dev) {
        w = (float2 *)psi;
    } else {
        CUDA_TRY(c, c->wave.ensure(wbytes));
        w = (float2 *)c->wave.p;
        if (!plane_wave) CUDA_TRY(c, cudaMemcpyAsync(w, psi, wbytes, cudaMemcpyHostToDevice, c->stream));
    }
    SliceTables st;
    if ((rc = build_slice_tables(c, g, o, ntrans, dz, st))) return rc;
    float2 *twr = twiddles(c, ny), *twc = twiddles(c, nx);
    if (!twr || !twc) return fail(c, MSL_E_NOMEM, "twiddle table allocation failed");
    const int colf = msl::COL_LOAD | msl::COL_FWD | msl::COL_PROP | msl::COL_INV | msl::COL_STORE;
    auto loop = [&]() -> int {
        for (int s = 0; s < nslice; ++s) {
            const int l = layer_seq[s];
            int rf = msl::ROW_TRANS | msl::ROW_FWD;
            if (s > 0) rf |= msl::ROW_LOAD | msl::ROW_INV;
            else if (!plane_wave) rf |= msl::ROW_LOAD;
            RowArgs r = row_args(g, twr, td + (size_t)l * n2, w, batch, rf, c->dflag);
            LAUNCH_TRY(c, timed(c, MSL_PROF_ROW, [&] { return msl::launch_row_pass(ny, r, c->stream, c->nsm, &c->launches); }));
            ColArgs ca = col_args(g, st, twc, l, w, batch, colf, c->dflag);
            LAUNCH_TRY(c, timed(c, MSL_PROF_COL, [&] { return msl::launch_col_pass(nx, ca, c->stream, c->nsm, &c->launches); }));
        }
        RowArgs r = row_args(g, twr, nullptr, w, batch, msl::ROW_LOAD | msl::ROW_INV, c->dflag);
        LAUNCH_TRY(c, timed(c, MSL_PROF_ROW, [&] { return msl::launch_row_pass(ny, r, c->stream, c->nsm, &c->launches); }));
        return MSL_OK;
    };
    // Small batches are launch-bound (a 256^2 wave's pass is a few microseconds):
    // their loop runs as one CUDA graph once the same call has been seen twice.
    // The tables the kernels read are uploaded above on every call; the graph
    // holds only launches.
    const bool graphable = !c->prof && wbytes <= ((size_t)32 << 20) && nslice >= 4;
    if (!graphable) {
        if ((rc = loop())) return rc;
    } else {
        std::vector<unsigned char> key;
        auto put = [&](const void *p, size_t n) {
            key.insert(key.end(), (const unsigned char *)p, (const unsigned char *)p + n);
        };
        int sch[4] = {0, 0, 0, 0};
        msl::get_schedule(nx, &sch[0], &sch[1]);
        msl::get_schedule(ny, &sch[2], &sch[3]);
        const void *ptrs[8] = {td, w, twr, twc, st.d_prop, st.d_kx2, st.d_ky2, c->dflag};
        const int ints[6] = {nx, ny, batch, nslice, plane_wave, ntrans};
        put(sch, sizeof(sch));
        put(ptrs, sizeof(ptrs));
        put(ints, sizeof(ints));
        put(&st.k2max, sizeof(st.k2max));
        put(&c->device, sizeof(c->device));
        put(layer_seq, sizeof(int) * (size_t)nslice);
        LoopGraphRun lg(c);
        if ((rc = lg.run(key, loop))) return rc;
    }
    if (!dev) CUDA_TRY(c, cudaMemcpyAsync(psi, w, wbytes, cudaMemcpyDeviceToHost, c->stream));
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    collect_profile(c);
    if (c->dflag && (rc = err_check(c))) return rc;
    return MSL_OK;
}

int msl_stem_scan(msl_ctx *c, const msl_grid *g, const msl_optics *o, const float *trans,
                  int ntrans, const double *dz, const int *layer_seq, int nslice,
                  const msl_probe *pr, const double *probe_xy, int nprobe,
                  const msl_detectors *det, const int *checkpoints, int ncheck, double *det_out) {
    if (!c) return MSL_E_ARG;
    int rc = check_grid(c, g);
    if (rc) return rc;
    if ((rc = check_optics(c, o))) return rc;
    if ((rc = check_layers(c, ntrans, dz, layer_seq, nslice))) return rc;
    if (!trans || !pr || !probe_xy || !det || !checkpoints || !det_out)
        return fail(c, MSL_E_ARG, "null argument");
    if (nprobe < 1) return fail(c, MSL_E_ARG, "nprobe must be >= 1");
    if (det->ndet < 1 || det->ndet > MSL_MAX_DETECTORS || !det->k_in || !det->k_out)
        return fail(c, MSL_E_ARG, "1..8 detectors with k_in/k_out arrays are required");
    for (int d = 0; d < det->ndet; ++d)
        if (!(det->k_in[d] >= 0) || !(det->k_out[d] >= det->k_in[d]) || !is_fin(det->k_out[d]))
            return fail(c, MSL_E_ARG, "detector bounds must satisfy 0 <= k_in <= k_out");
    if (!(pr->k_in >= 0) || !(pr->k_out > pr->k_in) || !is_fin(pr->k_out) || !is_fin(pr->df) ||
        !is_fin(pr->cs))
        return fail(c, MSL_E_ARG, "probe aperture must satisfy 0 <= k_in < k_out; df, cs finite");
    if (ncheck < 1) return fail(c, MSL_E_ARG, "ncheck must be >= 1");
    for (int i = 0; i < ncheck; ++i)
        if (checkpoints[i] < 0 || checkpoints[i] >= nslice || (i > 0 && checkpoints[i] <= checkpoints[i - 1]))
            return fail(c, MSL_E_ARG, "checkpoints must be ascending slice indices in [0, nslice)");
    for (int p = 0; p < 2 * nprobe; ++p)
        if (!is_fin(probe_xy[p])) return fail(c, MSL_E_ARG, "probe positions must be finite");
    CUDA_TRY(c, cudaSetDevice(c->device));
    if ((rc = maybe_tune(c, g->nx)) || (g->ny != g->nx && (rc = maybe_tune(c, g->ny)))) return rc;
    if ((rc = err_reset(c))) return rc;
    const int nx = g->nx, ny = g->ny, ndet = det->ndet;
    const size_t n2 = (size_t)nx * ny;
    int ntile = 0;  // column tiles per image of the column pass that will run (set below)
    const float2 *td;
    if ((rc = stage_in(c, (const float2 *)trans, sizeof(float2) * n2 * ntrans, c->trans_stage, &td)))
        return rc;
    SliceTables st;
    if ((rc = build_slice_tables(c, g, o, ntrans, dz, st))) return rc;
    float2 *twr = twiddles(c, ny), *twc = twiddles(c, nx);
    if (!twr || !twc) return fail(c, MSL_E_NOMEM, "twiddle table allocation failed");

    // reciprocal coordinates (double) of MSProject.cs:470-484 and detector bounds
    std::vector<double> hk(nx + ny + 2 * ndet);
    for (int i = 0; i < nx; ++i) hk[i] = (double)(i < nx / 2 ? i : i - nx) / g->ax;
    for (int i = 0; i < ny; ++i) hk[nx + i] = (double)(i < ny / 2 ? i : i - ny) / g->by;
    for (int d = 0; d < ndet; ++d) {
        hk[nx + ny + d] = det->k_in[d] * det->k_in[d];
        hk[nx + ny + ndet + d] = det->k_out[d] * det->k_out[d];
    }
    if ((rc = upload(c, c->fxy, hk.data(), sizeof(double) * hk.size()))) return rc;
    const double *kxd = (const double *)c->fxy.p, *kyd = kxd + nx;
    CUDA_TRY(c, c->apchi.ensure(sizeof(float2) * n2 + n2));
    float2 *apchi = (float2 *)c->apchi.p;
    uint8_t *mask = (uint8_t *)(apchi + n2);
    const double lam = msl_wavelength(o->kev);
    LAUNCH_TRY(c, timed(c, MSL_PROF_OTHER, [&] { return msl::launch_probe_table(nx, ny, kxd, kyd, pr->k_in * pr->k_in, pr->k_out * pr->k_out,
                                          lam, pr->df, pr->cs, 1.0 / ((double)nx * ny), apchi,
                                          c->stream, &c->launches); }));
    LAUNCH_TRY(c, timed(c, MSL_PROF_OTHER, [&] { return msl::launch_detector_mask(nx, ny, kxd, kyd, ndet, kyd + ny, kyd + ny + ndet, mask,
                                            c->stream, &c->launches); }));
    int B = c->probe_batch;
    if (B <= 0) {
        // wave buffer budget: 8 GiB, or half the context's memory cap when one is set
        size_t budget = (size_t)8 << 30;
        if (c->mem.limit && c->mem.limit / 2 < budget) budget = c->mem.limit / 2;
        B = (int)std::max<size_t>(1, std::min<size_t>(budget / (sizeof(float2) * n2), 65536));
    }
    if (B > nprobe) B = nprobe;
    CUDA_TRY(c, c->wave.ensure(sizeof(float2) * n2 * B));
    CUDA_TRY(c, c->exy.ensure(sizeof(float2) * (size_t)B * (nx + ny) + sizeof(double) * 2 * B));
    const size_t obytes = sizeof(double) * (size_t)nprobe * ncheck * ndet;
    const bool odev = on_device(det_out);
    double *od;
    if (odev) {
        od = det_out;
    } else {
        CUDA_TRY(c, c->detout.ensure(obytes));
        od = (double *)c->detout.p;
    }
    float2 *w = (float2 *)c->wave.p;
    {
        ColArgs probe_cfg = col_args(g, st, twc, 0, w, 1, msl::COL_LOAD | msl::COL_STORE, c->dflag);
        ntile = ny / msl::plan_col_c_launch(nx, probe_cfg);
    }
    CUDA_TRY(c, c->partial.ensure(sizeof(double) * (size_t)ncheck * B * ntile * ndet));
    float2 *ex = (float2 *)c->exy.p, *ey = ex + (size_t)B * nx;
    double *fxy = (double *)(ey + (size_t)B * ny);
    double *partial = (double *)c->partial.p;
    const int last = checkpoints[ncheck - 1];
    std::vector<double> hf(2 * (size_t)B);
    const double dscale = (double)n2 * (double)n2;
    for (int p0 = 0; p0 < nprobe; p0 += B) {
        const int nb = std::min(B, nprobe - p0);
        for (int b = 0; b < nb; ++b) {
            hf[2 * b] = probe_xy[2 * (p0 + b)] / g->ax;
            hf[2 * b + 1] = probe_xy[2 * (p0 + b) + 1] / g->by;
        }
        CUDA_TRY(c, cudaMemcpyAsync(fxy, hf.data(), sizeof(double) * 2 * nb, cudaMemcpyHostToDevice,
                                    c->stream));
        LAUNCH_TRY(c, timed(c, MSL_PROF_OTHER, [&] { return msl::launch_probe_shifts(nx, ny, nb, fxy, ex, ey, c->stream, &c->launches); }));
        ColArgs pa = col_args(g, st, twc, 0, w, nb, msl::COL_PROBE | msl::COL_INV | msl::COL_STORE, c->dflag);
        pa.apchi = apchi;
        pa.ex = ex;
        pa.ey = ey;
        LAUNCH_TRY(c, timed(c, MSL_PROF_COL, [&] { return msl::launch_col_pass(nx, pa, c->stream, c->nsm, &c->launches); }));
        int ic = 0;
        for (int s = 0; s <= last; ++s) {
            const int l = layer_seq[s];
            RowArgs r = row_args(g, twr, td + (size_t)l * n2, w, nb, msl::ROW_LOAD | msl::ROW_INV | msl::ROW_TRANS | msl::ROW_FWD, c->dflag);
            LAUNCH_TRY(c, timed(c, MSL_PROF_ROW, [&] { return msl::launch_row_pass(ny, r, c->stream, c->nsm, &c->launches); }));
            const bool detect = checkpoints[ic] == s;
            int cf = msl::COL_LOAD | msl::COL_FWD | msl::COL_PROP;
            if (detect) cf |= msl::COL_DETECT;
            if (s < last) cf |= msl::COL_INV | msl::COL_STORE;
            ColArgs ca = col_args(g, st, twc, l, w, nb, cf, c->dflag);
            ca.detmask = mask;
            ca.ndet = ndet;
            ca.partial = partial + (size_t)ic * B * ntile * ndet;
            LAUNCH_TRY(c, timed(c, MSL_PROF_COL, [&] { return msl::launch_col_pass(nx, ca, c->stream, c->nsm, &c->launches); }));
            if (detect) {
                LAUNCH_TRY(c, timed(c, MSL_PROF_OTHER, [&] { return msl::launch_detector_finalize(
                                  nb, ntile, ndet, ca.partial, dscale,
                                  od + ((size_t)p0 * ncheck + ic) * ndet, ncheck * ndet, c->stream,
                                  &c->launches); }));
                ++ic;
            }
        }
    }
    if (!odev) CUDA_TRY(c, cudaMemcpyAsync(det_out, od, obytes, cudaMemcpyDeviceToHost, c->stream));
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    collect_profile(c);
    if (c->dflag && (rc = err_check(c))) return rc;
    return MSL_OK;
}

int msl_tc_gemm_bf16(msl_ctx *c, const uint16_t *A, const uint16_t *B, float *D, int M, int N, int K) {
    if (!c) return MSL_E_ARG;
    if (!A || !B || !D) return fail(c, MSL_E_ARG, "null argument");
    if (M <= 0 || M % 128 || K <= 0 || K % 64 || N < 16 || N > 256 || N % 16)
        return fail(c, MSL_E_ARG, "M % 128 == 0, K % 64 == 0, 16 <= N <= 256, N % 16 == 0 required");
    CUDA_TRY(c, cudaSetDevice(c->device));
    int rc;
    if ((rc = err_reset(c))) return rc;
    const uint16_t *ad, *bd;
    if ((rc = stage_in(c, A, sizeof(uint16_t) * (size_t)M * K, c->in_stage, &ad))) return rc;
    if ((rc = stage_in(c, B, sizeof(uint16_t) * (size_t)N * K, c->trans_stage, &bd))) return rc;
    const bool ddev = on_device(D);
    float *dd = D;
    if (!ddev) {
        CUDA_TRY(c, c->tmpw.ensure(sizeof(float) * (size_t)M * N));
        dd = (float *)c->tmpw.p;
    }
    LAUNCH_TRY(c, timed(c, MSL_PROF_OTHER, [&] {
                   return msl::launch_tc_gemm(ad, bd, dd, M, N, K, c->dflag, c->stream, &c->launches);
               }));
    if (!ddev) CUDA_TRY(c, cudaMemcpyAsync(D, dd, sizeof(float) * (size_t)M * N, cudaMemcpyDeviceToHost, c->stream));
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    collect_profile(c);
    if ((rc = err_check(c))) return rc;
    return MSL_OK;
}

}  // extern "C"

struct msl_closure {
    int device = 0;
    msl::ClosureNet net;
};

namespace {

int closure_check(msl_ctx *c, const msl_closure *n, int batch, int h, int w) {
    if (!c || !n) return MSL_E_ARG;
    if (n->device != c->device) return fail(c, MSL_E_ARG, "closure and context are on different devices");
    if (batch < 1 || h < 3 || w < 128 || w % 128)
        return fail(c, MSL_E_ARG, "closure images need batch >= 1, height >= 3 and a width that is a multiple of 128");
    return MSL_OK;
}

// Sum of the forward pass's per-block loss terms / pixel count (after a sync).
int closure_loss(msl_ctx *c, msl_closure *n, size_t npix, double *loss) {
    if (!loss) return MSL_OK;
    std::vector<double> part(n->net.loss_blocks);
    CUDA_TRY(c, cudaMemcpy(part.data(), n->net.loss_part, sizeof(double) * part.size(), cudaMemcpyDeviceToHost));
    double s = 0.0;
    for (double v : part) s += v;
    *loss = s / (double)npix;
    return MSL_OK;
}

}  // namespace

extern "C" {

int msl_closure_param_count(void) { return msl::closure_param_count(); }

int msl_closure_create(msl_ctx *c, uint64_t seed, msl_closure **out) {
    if (!c || !out) return MSL_E_ARG;
    CUDA_TRY(c, cudaSetDevice(c->device));
    msl_closure *n = new msl_closure();
    n->device = c->device;
    if (n->net.alloc_params() != cudaSuccess) {
        n->net.release();
        delete n;
        cudaGetLastError();
        return fail(c, MSL_E_NOMEM, "closure parameter allocation failed");
    }
    std::vector<float> h;
    msl::closure_init_params(seed, h);
    if (cudaMemcpy(n->net.params, h.data(), sizeof(float) * h.size(), cudaMemcpyHostToDevice) != cudaSuccess) {
        n->net.release();
        delete n;
        return fail(c, MSL_E_CUDA, "closure parameter upload failed");
    }
    *out = n;
    return MSL_OK;
}

int msl_closure_destroy(msl_closure *n) {
    if (!n) return MSL_E_ARG;
    int cur = 0;
    cudaGetDevice(&cur);
    cudaSetDevice(n->device);
    n->net.release();
    cudaSetDevice(cur);
    delete n;
    return MSL_OK;
}

int msl_closure_get_params(msl_ctx *c, const msl_closure *n, float *out) {
    if (!c || !n || !out) return MSL_E_ARG;
    CUDA_TRY(c, cudaSetDevice(c->device));
    CUDA_TRY(c, cudaMemcpy(out, n->net.params, sizeof(float) * msl::closure_param_count(), cudaMemcpyDefault));
    return MSL_OK;
}

int msl_closure_set_params(msl_ctx *c, msl_closure *n, const float *in) {
    if (!c || !n || !in) return MSL_E_ARG;
    CUDA_TRY(c, cudaSetDevice(c->device));
    const size_t b = sizeof(float) * msl::closure_param_count();
    CUDA_TRY(c, cudaMemcpy(n->net.params, in, b, cudaMemcpyDefault));
    CUDA_TRY(c, cudaMemset(n->net.adam_m, 0, b));
    CUDA_TRY(c, cudaMemset(n->net.adam_v, 0, b));
    n->net.step = 0;
    return MSL_OK;
}

int msl_closure_apply(msl_ctx *c, msl_closure *n, float *psi, int batch, int h, int w) {
    int rc = closure_check(c, n, batch, h, w);
    if (rc) return rc;
    if (!psi) return fail(c, MSL_E_ARG, "psi is null");
    CUDA_TRY(c, cudaSetDevice(c->device));
    if ((rc = err_reset(c))) return rc;
    const size_t bytes = sizeof(float2) * (size_t)batch * h * w;
    const float2 *pd;
    if ((rc = stage_in(c, (const float2 *)psi, bytes, c->in_stage, &pd))) return rc;
    float2 *io = (float2 *)pd;
    LAUNCH_TRY(c, timed(c, MSL_PROF_OTHER, [&] {
                   return n->net.forward(io, batch, h, w, io, nullptr, false, c->dflag, c->stream, c->nsm,
                                         &c->launches);
               }));
    if ((const void *)io != (const void *)psi)
        CUDA_TRY(c, cudaMemcpyAsync(psi, io, bytes, cudaMemcpyDeviceToHost, c->stream));
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    collect_profile(c);
    return err_check(c);
}

// Shared by msl_closure_gradients and msl_closure_train_step.
static int closure_fwd_bwd(msl_ctx *c, msl_closure *n, const float *coarse, const float *fine, int batch, int h,
                           int w, double *loss) {
    int rc = closure_check(c, n, batch, h, w);
    if (rc) return rc;
    if (!coarse || !fine) return fail(c, MSL_E_ARG, "coarse and fine waves are required");
    CUDA_TRY(c, cudaSetDevice(c->device));
    if ((rc = err_reset(c))) return rc;
    const size_t npix = (size_t)batch * h * w, bytes = sizeof(float2) * npix;
    const float2 *cd, *fd;
    if ((rc = stage_in(c, (const float2 *)coarse, bytes, c->in_stage, &cd))) return rc;
    if ((rc = stage_in(c, (const float2 *)fine, bytes, c->trans_stage, &fd))) return rc;
    LAUNCH_TRY(c, timed(c, MSL_PROF_OTHER, [&] {
                   return n->net.forward(cd, batch, h, w, nullptr, fd, true, c->dflag, c->stream, c->nsm,
                                         &c->launches);
               }));
    LAUNCH_TRY(c, timed(c, MSL_PROF_OTHER, [&] {
                   return n->net.backward(batch, h, w, c->dflag, c->stream, c->nsm, &c->launches);
               }));
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    if ((rc = closure_loss(c, n, npix, loss))) return rc;
    return MSL_OK;
}

int msl_closure_gradients(msl_ctx *c, msl_closure *n, const float *coarse, const float *fine, int batch, int h,
                          int w, float *grad, double *loss) {
    int rc = closure_fwd_bwd(c, n, coarse, fine, batch, h, w, loss);
    if (rc) return rc;
    if (grad)
        CUDA_TRY(c, cudaMemcpy(grad, n->net.grads, sizeof(float) * msl::closure_param_count(), cudaMemcpyDefault));
    collect_profile(c);
    return err_check(c);
}

int msl_closure_train_step(msl_ctx *c, msl_closure *n, const float *coarse, const float *fine, int batch, int h,
                           int w, float lr, double *loss) {
    if (!(lr > 0) || !is_fin(lr)) return fail(c, MSL_E_ARG, "learning rate must be positive");
    int rc = closure_fwd_bwd(c, n, coarse, fine, batch, h, w, loss);
    if (rc) return rc;
    LAUNCH_TRY(c, n->net.adam(lr, c->stream, c->nsm, &c->launches));
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    collect_profile(c);
    return err_check(c);
}

}  // extern "C"

namespace {

// Shared set-up of the exit-wave scans (msl_stem_exit_waves, msl_stem_scan_closure):
// slice tables of ntrans layers plus an identity layer (index ntrans: band limit
// and the 1/(nx ny) scale only), twiddles, the probe table and, when det is given,
// the detector mask; work buffers for B probes.
struct ExitScan {
    SliceTables st;
    float2 *twr = nullptr, *twc = nullptr;
    const float2 *td = nullptr;
    float2 *apchi = nullptr, *ex = nullptr, *ey = nullptr, *w = nullptr;
    uint8_t *mask = nullptr;
    double *fxy = nullptr, *partial = nullptr;
    int B = 0, ntile = 0, ntrans = 0;
};

int exit_scan_setup(msl_ctx *c, const msl_grid *g, const msl_optics *o, const float *trans, int ntrans,
                    const double *dz, const msl_probe *pr, const msl_detectors *det, int nprobe, size_t max_b,
                    ExitScan &X) {
    const int nx = g->nx, ny = g->ny, ndet = det ? det->ndet : 0;
    const size_t n2 = (size_t)nx * ny;
    int rc;
    if ((rc = stage_in(c, (const float2 *)trans, sizeof(float2) * n2 * ntrans, c->trans_stage, &X.td))) return rc;
    std::vector<double> dze(dz, dz + ntrans);
    dze.push_back(0.0);  // the identity layer
    if ((rc = build_slice_tables(c, g, o, ntrans + 1, dze.data(), X.st))) return rc;
    X.ntrans = ntrans;
    X.twr = twiddles(c, ny);
    X.twc = twiddles(c, nx);
    if (!X.twr || !X.twc) return fail(c, MSL_E_NOMEM, "twiddle table allocation failed");
    std::vector<double> hk(nx + ny + 2 * ndet);
    for (int i = 0; i < nx; ++i) hk[i] = (double)(i < nx / 2 ? i : i - nx) / g->ax;
    for (int i = 0; i < ny; ++i) hk[nx + i] = (double)(i < ny / 2 ? i : i - ny) / g->by;
    for (int d = 0; d < ndet; ++d) {
        hk[nx + ny + d] = det->k_in[d] * det->k_in[d];
        hk[nx + ny + ndet + d] = det->k_out[d] * det->k_out[d];
    }
    if ((rc = upload(c, c->fxy, hk.data(), sizeof(double) * hk.size()))) return rc;
    const double *kxd = (const double *)c->fxy.p, *kyd = kxd + nx;
    CUDA_TRY(c, c->apchi.ensure(sizeof(float2) * n2 + n2));
    X.apchi = (float2 *)c->apchi.p;
    X.mask = (uint8_t *)(X.apchi + n2);
    const double lam = msl_wavelength(o->kev);
    LAUNCH_TRY(c, timed(c, MSL_PROF_OTHER, [&] {
                   return msl::launch_probe_table(nx, ny, kxd, kyd, pr->k_in * pr->k_in, pr->k_out * pr->k_out, lam,
                                                  pr->df, pr->cs, 1.0 / ((double)nx * ny), X.apchi, c->stream,
                                                  &c->launches);
               }));
    if (det)
        LAUNCH_TRY(c, timed(c, MSL_PROF_OTHER, [&] {
                       return msl::launch_detector_mask(nx, ny, kxd, kyd, ndet, kyd + ny, kyd + ny + ndet, X.mask,
                                                        c->stream, &c->launches);
                   }));
    int B = c->probe_batch;
    if (B <= 0) {
        size_t budget = (size_t)8 << 30;
        if (c->mem.limit && c->mem.limit / 2 < budget) budget = c->mem.limit / 2;
        B = (int)std::max<size_t>(1, std::min<size_t>(budget / (sizeof(float2) * n2), 65536));
    }
    if ((size_t)B > max_b) B = (int)max_b;
    if (B > nprobe) B = nprobe;
    X.B = B;
    CUDA_TRY(c, c->wave.ensure(sizeof(float2) * n2 * B));
    CUDA_TRY(c, c->exy.ensure(sizeof(float2) * (size_t)B * (nx + ny) + sizeof(double) * 2 * B));
    X.w = (float2 *)c->wave.p;
    X.ex = (float2 *)c->exy.p;
    X.ey = X.ex + (size_t)B * nx;
    X.fxy = (double *)(X.ey + (size_t)B * ny);
    if (det) {
        ColArgs probe_cfg = col_args(g, X.st, X.twc, 0, X.w, 1, msl::COL_LOAD | msl::COL_STORE, c->dflag);
        X.ntile = ny / msl::plan_col_c_launch(nx, probe_cfg);
        CUDA_TRY(c, c->partial.ensure(sizeof(double) * (size_t)B * X.ntile * ndet));
        X.partial = (double *)c->partial.p;
    }
    return MSL_OK;
}

// Probes p0 .. p0 + nb - 1 through the slice loop: X.w receives their real-space exit waves.
int exit_scan_batch(msl_ctx *c, const msl_grid *g, ExitScan &X, const int *layer_seq, int nslice,
                    const double *probe_xy, int p0, int nb) {
    const int nx = g->nx, ny = g->ny;
    std::vector<double> hf(2 * (size_t)nb);
    for (int b = 0; b < nb; ++b) {
        hf[2 * b] = probe_xy[2 * (p0 + b)] / g->ax;
        hf[2 * b + 1] = probe_xy[2 * (p0 + b) + 1] / g->by;
    }
    CUDA_TRY(c, cudaMemcpyAsync(X.fxy, hf.data(), sizeof(double) * 2 * nb, cudaMemcpyHostToDevice, c->stream));
    LAUNCH_TRY(c, timed(c, MSL_PROF_OTHER, [&] {
                   return msl::launch_probe_shifts(nx, ny, nb, X.fxy, X.ex, X.ey, c->stream, &c->launches);
               }));
    ColArgs pa = col_args(g, X.st, X.twc, 0, X.w, nb, msl::COL_PROBE | msl::COL_INV | msl::COL_STORE, c->dflag);
    pa.apchi = X.apchi;
    pa.ex = X.ex;
    pa.ey = X.ey;
    LAUNCH_TRY(c, timed(c, MSL_PROF_COL, [&] { return msl::launch_col_pass(nx, pa, c->stream, c->nsm, &c->launches); }));
    const size_t n2 = (size_t)nx * ny;
    for (int s = 0; s < nslice; ++s) {
        const int l = layer_seq[s];
        RowArgs r = row_args(g, X.twr, X.td + (size_t)l * n2, X.w, nb,
                             msl::ROW_LOAD | msl::ROW_INV | msl::ROW_TRANS | msl::ROW_FWD, c->dflag);
        LAUNCH_TRY(c, timed(c, MSL_PROF_ROW, [&] { return msl::launch_row_pass(ny, r, c->stream, c->nsm, &c->launches); }));
        ColArgs ca = col_args(g, X.st, X.twc, l, X.w, nb,
                              msl::COL_LOAD | msl::COL_FWD | msl::COL_PROP | msl::COL_INV | msl::COL_STORE, c->dflag);
        LAUNCH_TRY(c, timed(c, MSL_PROF_COL, [&] { return msl::launch_col_pass(nx, ca, c->stream, c->nsm, &c->launches); }));
    }
    RowArgs r = row_args(g, X.twr, nullptr, X.w, nb, msl::ROW_LOAD | msl::ROW_INV, c->dflag);
    LAUNCH_TRY(c, timed(c, MSL_PROF_ROW, [&] { return msl::launch_row_pass(ny, r, c->stream, c->nsm, &c->launches); }));
    return MSL_OK;
}

int exit_scan_check(msl_ctx *c, const msl_grid *g, const msl_optics *o, const float *trans, int ntrans,
                    const double *dz, const int *layer_seq, int nslice, const msl_probe *pr, const double *probe_xy,
                    int nprobe) {
    int rc = check_grid(c, g);
    if (rc) return rc;
    if ((rc = check_optics(c, o))) return rc;
    if ((rc = check_layers(c, ntrans, dz, layer_seq, nslice))) return rc;
    if (!trans || !pr || !probe_xy) return fail(c, MSL_E_ARG, "null argument");
    if (nprobe < 1) return fail(c, MSL_E_ARG, "nprobe must be >= 1");
    if (!(pr->k_in >= 0) || !(pr->k_out > pr->k_in) || !is_fin(pr->k_out) || !is_fin(pr->df) || !is_fin(pr->cs))
        return fail(c, MSL_E_ARG, "probe aperture must satisfy 0 <= k_in < k_out; df, cs finite");
    for (int p = 0; p < 2 * nprobe; ++p)
        if (!is_fin(probe_xy[p])) return fail(c, MSL_E_ARG, "probe positions must be finite");
    return MSL_OK;
}

}  // namespace

extern "C" {

int msl_stem_exit_waves(msl_ctx *c, const msl_grid *g, const msl_optics *o, const float *trans, int ntrans,
                        const double *dz, const int *layer_seq, int nslice, const msl_probe *pr,
                        const double *probe_xy, int nprobe, float *psi_out) {
    if (!c) return MSL_E_ARG;
    int rc = exit_scan_check(c, g, o, trans, ntrans, dz, layer_seq, nslice, pr, probe_xy, nprobe);
    if (rc) return rc;
    if (!psi_out) return fail(c, MSL_E_ARG, "psi_out is null");
    CUDA_TRY(c, cudaSetDevice(c->device));
    if ((rc = err_reset(c))) return rc;
    ExitScan X;
    if ((rc = exit_scan_setup(c, g, o, trans, ntrans, dz, pr, nullptr, nprobe, (size_t)nprobe, X))) return rc;
    const size_t n2 = (size_t)g->nx * g->ny;
    for (int p0 = 0; p0 < nprobe; p0 += X.B) {
        const int nb = std::min(X.B, nprobe - p0);
        if ((rc = exit_scan_batch(c, g, X, layer_seq, nslice, probe_xy, p0, nb))) return rc;
        CUDA_TRY(c, cudaMemcpyAsync(psi_out + 2 * n2 * p0, X.w, sizeof(float2) * n2 * nb, cudaMemcpyDefault,
                                    c->stream));
        CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    }
    collect_profile(c);
    return err_check(c);
}

int msl_stem_scan_closure(msl_ctx *c, msl_closure *n, const msl_grid *g, const msl_optics *o, const float *trans,
                          int ntrans, const double *dz, const int *layer_seq, int nslice, const msl_probe *pr,
                          const double *probe_xy, int nprobe, const msl_detectors *det, double *det_out) {
    if (!c || !n) return MSL_E_ARG;
    int rc = exit_scan_check(c, g, o, trans, ntrans, dz, layer_seq, nslice, pr, probe_xy, nprobe);
    if (rc) return rc;
    if (n->device != c->device) return fail(c, MSL_E_ARG, "closure and context are on different devices");
    if (g->ny % 128) return fail(c, MSL_E_ARG, "the closure needs ny to be a multiple of 128");
    if (!det || !det_out || det->ndet < 1 || det->ndet > MSL_MAX_DETECTORS || !det->k_in || !det->k_out)
        return fail(c, MSL_E_ARG, "1..8 detectors with k_in/k_out arrays and det_out are required");
    for (int d = 0; d < det->ndet; ++d)
        if (!(det->k_in[d] >= 0) || !(det->k_out[d] >= det->k_in[d]) || !is_fin(det->k_out[d]))
            return fail(c, MSL_E_ARG, "detector bounds must satisfy 0 <= k_in <= k_out");
    CUDA_TRY(c, cudaSetDevice(c->device));
    if ((rc = err_reset(c))) return rc;
    const int nx = g->nx, ny = g->ny, ndet = det->ndet;
    const size_t n2 = (size_t)nx * ny;
    // the closure keeps two bf16 activation planes of 64 channels per pixel: its
    // sub-batch is sized to 4 GiB of them, the wave batch to a whole number of those
    const int CB = (int)std::max<size_t>(1, ((size_t)4 << 30) / (256 * n2));
    ExitScan X;
    if ((rc = exit_scan_setup(c, g, o, trans, ntrans, dz, pr, det, nprobe, (size_t)1 << 30, X))) return rc;
    const size_t obytes = sizeof(double) * (size_t)nprobe * ndet;
    const bool odev = on_device(det_out);
    double *od;
    if (odev) {
        od = det_out;
    } else {
        CUDA_TRY(c, c->detout.ensure(obytes));
        od = (double *)c->detout.p;
    }
    const double dscale = (double)n2 * (double)n2;
    for (int p0 = 0; p0 < nprobe; p0 += X.B) {
        const int nb = std::min(X.B, nprobe - p0);
        if ((rc = exit_scan_batch(c, g, X, layer_seq, nslice, probe_xy, p0, nb))) return rc;
        for (int b0 = 0; b0 < nb; b0 += CB) {
            const int cb = std::min(CB, nb - b0);
            float2 *wb = X.w + n2 * b0;
            LAUNCH_TRY(c, timed(c, MSL_PROF_OTHER, [&] {
                           return n->net.forward(wb, cb, nx, ny, wb, nullptr, false, c->dflag, c->stream, c->nsm,
                                                 &c->launches);
                       }));
        }
        // forward transform of the corrected exit waves and detection inside the band limit
        RowArgs r = row_args(g, X.twr, nullptr, X.w, nb, msl::ROW_LOAD | msl::ROW_FWD, c->dflag);
        LAUNCH_TRY(c, timed(c, MSL_PROF_ROW, [&] { return msl::launch_row_pass(ny, r, c->stream, c->nsm, &c->launches); }));
        ColArgs ca = col_args(g, X.st, X.twc, X.ntrans, X.w, nb, msl::COL_LOAD | msl::COL_FWD | msl::COL_PROP | msl::COL_DETECT,
                              c->dflag);
        ca.detmask = X.mask;
        ca.ndet = ndet;
        ca.partial = X.partial;
        LAUNCH_TRY(c, timed(c, MSL_PROF_COL, [&] { return msl::launch_col_pass(nx, ca, c->stream, c->nsm, &c->launches); }));
        LAUNCH_TRY(c, timed(c, MSL_PROF_OTHER, [&] {
                       return msl::launch_detector_finalize(nb, X.ntile, ndet, X.partial, dscale, od + (size_t)p0 * ndet,
                                                            ndet, c->stream, &c->launches);
                   }));
    }
    if (!odev) CUDA_TRY(c, cudaMemcpyAsync(det_out, od, obytes, cudaMemcpyDeviceToHost, c->stream));
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    collect_profile(c);
    return err_check(c);
}

int msl_stem_scan_resident(msl_ctx *c, const msl_grid *g, const msl_optics *o, const float *trans, int ntrans,
                           const double *dz, const int *layer_seq, int nslice, const msl_probe *pr,
                           const double *probe_xy, int nprobe, const msl_detectors *det, const int *checkpoints,
                           int ncheck, double *det_out) {
    if (!c) return MSL_E_ARG;
    int rc = exit_scan_check(c, g, o, trans, ntrans, dz, layer_seq, nslice, pr, probe_xy, nprobe);
    if (rc) return rc;
    const int side = msl::resident_side();
    if (g->nx != side || g->ny != side)
        return fail(c, MSL_E_UNSUPPORTED, "the resident slice loop is built for " + std::to_string(side) + "^2 grids");
    if (!det || !det_out || !checkpoints || det->ndet < 1 || det->ndet > MSL_MAX_DETECTORS || !det->k_in || !det->k_out)
        return fail(c, MSL_E_ARG, "1..8 detectors with k_in/k_out arrays, checkpoints and det_out are required");
    for (int d = 0; d < det->ndet; ++d)
        if (!(det->k_in[d] >= 0) || !(det->k_out[d] >= det->k_in[d]) || !is_fin(det->k_out[d]))
            return fail(c, MSL_E_ARG, "detector bounds must satisfy 0 <= k_in <= k_out");
    if (ncheck < 1) return fail(c, MSL_E_ARG, "ncheck must be >= 1");
    for (int i = 0; i < ncheck; ++i)
        if (checkpoints[i] < 0 || checkpoints[i] >= nslice || (i > 0 && checkpoints[i] <= checkpoints[i - 1]))
            return fail(c, MSL_E_ARG, "checkpoints must be ascending slice indices in [0, nslice)");
    CUDA_TRY(c, cudaSetDevice(c->device));
    if ((rc = err_reset(c))) return rc;
    const int ndet = det->ndet, ncl = msl::resident_cluster();
    const size_t n2 = (size_t)side * side;
    ExitScan X;
    if ((rc = exit_scan_setup(c, g, o, trans, ntrans, dz, pr, det, nprobe, (size_t)nprobe, X))) return rc;
    // device copies of the slice sequence and checkpoints
    std::vector<int> seqc(nslice + ncheck);
    for (int s2 = 0; s2 < nslice; ++s2) seqc[s2] = layer_seq[s2];
    for (int i = 0; i < ncheck; ++i) seqc[nslice + i] = checkpoints[i];
    if ((rc = upload(c, c->jobtab, seqc.data(), sizeof(int) * seqc.size()))) return rc;
    const int *dseq = (const int *)c->jobtab.p;
    CUDA_TRY(c, c->partial.ensure(sizeof(double) * (size_t)ncheck * X.B * ncl * ndet));
    double *partial = (double *)c->partial.p;
    const size_t obytes = sizeof(double) * (size_t)nprobe * ncheck * ndet;
    const bool odev = on_device(det_out);
    double *od;
    if (odev) {
        od = det_out;
    } else {
        CUDA_TRY(c, c->detout.ensure(obytes));
        od = (double *)c->detout.p;
    }
    const double dscale = (double)n2 * (double)n2;
    std::vector<double> hf(2 * (size_t)X.B);
    for (int p0 = 0; p0 < nprobe; p0 += X.B) {
        const int nb = std::min(X.B, nprobe - p0);
        for (int b = 0; b < nb; ++b) {
            hf[2 * b] = probe_xy[2 * (p0 + b)] / g->ax;
            hf[2 * b + 1] = probe_xy[2 * (p0 + b) + 1] / g->by;
        }
        CUDA_TRY(c, cudaMemcpyAsync(X.fxy, hf.data(), sizeof(double) * 2 * nb, cudaMemcpyHostToDevice, c->stream));
        LAUNCH_TRY(c, timed(c, MSL_PROF_OTHER, [&] {
                       return msl::launch_probe_shifts(side, side, nb, X.fxy, X.ex, X.ey, c->stream, &c->launches);
                   }));
        ColArgs pa = col_args(g, X.st, X.twc, 0, X.w, nb, msl::COL_PROBE | msl::COL_INV | msl::COL_STORE, c->dflag);
        pa.apchi = X.apchi;
        pa.ex = X.ex;
        pa.ey = X.ey;
        LAUNCH_TRY(c, timed(c, MSL_PROF_COL, [&] { return msl::launch_col_pass(side, pa, c->stream, c->nsm, &c->launches); }));
        msl::ResidentArgs ra;
        ra.w0 = X.w;
        ra.trans = X.td;
        ra.prop = X.st.d_prop;
        ra.kx2 = X.st.d_kx2;
        ra.ky2 = X.st.d_ky2;
        ra.k2max = X.st.k2max;
        ra.mask = X.mask;
        ra.ndet = ndet;
        ra.layer_seq = dseq;
        ra.nslice = nslice;
        ra.checkpoints = dseq + nslice;
        ra.ncheck = ncheck;
        ra.partial = partial;
        ra.nprobe = nb;
        ra.err = c->dflag;
        LAUNCH_TRY(c, timed(c, MSL_PROF_ROW, [&] { return msl::launch_stem_resident(ra, c->stream, c->nsm, &c->launches); }));
        for (int ic = 0; ic < ncheck; ++ic)
            LAUNCH_TRY(c, timed(c, MSL_PROF_OTHER, [&] {
                           return msl::launch_detector_finalize(nb, ncl, ndet, partial + (size_t)ic * nb * ncl * ndet,
                                                                dscale, od + ((size_t)p0 * ncheck + ic) * ndet,
                                                                ncheck * ndet, c->stream, &c->launches);
                       }));
    }
    if (!odev) CUDA_TRY(c, cudaMemcpyAsync(det_out, od, obytes, cudaMemcpyDeviceToHost, c->stream));
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    collect_profile(c);
    return err_check(c);
}

int msl_stem_scan_phonon(msl_ctx *c, const msl_atoms *at, const double *fparams, const msl_grid *g,
                         int nslice, double radius, const msl_optics *o, const msl_probe *pr,
                         const double *probe_xy, int nprobe, const msl_detectors *det,
                         const int *checkpoints, int ncheck, int nconfig, double sigma, uint64_t seed,
                         double *det_out) {
    if (!c) return MSL_E_ARG;
    int rc = check_grid(c, g);
    if (rc) return rc;
    if ((rc = check_optics(c, o))) return rc;
    if (!at || !fparams || !pr || !probe_xy || !det || !checkpoints || !det_out)
        return fail(c, MSL_E_ARG, "null argument");
    if (nconfig < 1 || !(sigma >= 0) || !is_fin(sigma) || nslice < 1 || nprobe < 1)
        return fail(c, MSL_E_ARG, "nconfig >= 1, sigma >= 0, nslice >= 1 and nprobe >= 1 are required");
    if (!(at->cz > 0) || !is_fin(at->cz)) return fail(c, MSL_E_ARG, "thickness cz must be positive");
    if (det->ndet < 1 || det->ndet > MSL_MAX_DETECTORS || !det->k_in || !det->k_out)
        return fail(c, MSL_E_ARG, "1..8 detectors with k_in/k_out arrays are required");
    for (int d = 0; d < det->ndet; ++d)
        if (!(det->k_in[d] >= 0) || !(det->k_out[d] >= det->k_in[d]) || !is_fin(det->k_out[d]))
            return fail(c, MSL_E_ARG, "detector bounds must satisfy 0 <= k_in <= k_out");
    if (!(pr->k_in >= 0) || !(pr->k_out > pr->k_in) || !is_fin(pr->k_out) || !is_fin(pr->df) ||
        !is_fin(pr->cs))
        return fail(c, MSL_E_ARG, "probe aperture must satisfy 0 <= k_in < k_out; df, cs finite");
    if (ncheck < 1) return fail(c, MSL_E_ARG, "ncheck must be >= 1");
    for (int i = 0; i < ncheck; ++i)
        if (checkpoints[i] < 0 || checkpoints[i] >= nslice || (i > 0 && checkpoints[i] <= checkpoints[i - 1]))
            return fail(c, MSL_E_ARG, "checkpoints must be ascending slice indices in [0, nslice)");
    for (int p = 0; p < 2 * nprobe; ++p)
        if (!is_fin(probe_xy[p])) return fail(c, MSL_E_ARG, "probe positions must be finite");
    CUDA_TRY(c, cudaSetDevice(c->device));
    const int nx = g->nx, ny = g->ny, ndet = det->ndet;
    const size_t n2 = (size_t)nx * ny;

    // configurations per batch: as many transmission stacks as 16 GiB hold (half
    // the context's cap when one is set); probes per launch then share the wave
    // budget (8 GiB, or a quarter of the cap) with them: images = configs x probes
    const size_t slab = sizeof(float2) * n2 * nslice;
    size_t tbudget = (size_t)16 << 30, wbudget = (size_t)8 << 30;
    if (c->mem.limit && c->mem.limit / 2 < tbudget) tbudget = c->mem.limit / 2;
    if (c->mem.limit && c->mem.limit / 4 < wbudget) wbudget = c->mem.limit / 4;
    const int BC = (int)std::max<size_t>(1, std::min<size_t>((size_t)nconfig, tbudget / slab));
    int BP = c->probe_batch > 0 ? c->probe_batch
                                : (int)std::max<size_t>(1, wbudget / (sizeof(float2) * n2 * BC));
    if (BP > nprobe) BP = nprobe;
    const int BI = BC * BP;  // images per launch at most
    DevBuf tbuf, pbuf;
    tbuf.mb = pbuf.mb = &c->mem;
    CUDA_TRY(c, tbuf.ensure(slab * BC));
    CUDA_TRY(c, pbuf.ensure(sizeof(float2 *) * (size_t)nslice * BI));

    std::vector<double> dz(nslice, at->cz / nslice);
    CUDA_TRY(c, c->wave.ensure(sizeof(float2) * n2 * BI));
    CUDA_TRY(c, c->exy.ensure(sizeof(float2) * (size_t)BI * (nx + ny) + sizeof(double) * 2 * BI));
    const size_t obytes = sizeof(double) * (size_t)nprobe * ncheck * ndet;
    const bool odev = on_device(det_out);
    double *od;
    if (odev) {
        od = det_out;
    } else {
        CUDA_TRY(c, c->detout.ensure(obytes));
        od = (double *)c->detout.p;
    }
    CUDA_TRY(c, cudaMemsetAsync(od, 0, obytes, c->stream));  // sums over configurations start at 0
    float2 *w = (float2 *)c->wave.p;
    float2 *ex = (float2 *)c->exy.p, *ey = ex + (size_t)BI * nx;
    double *fxy = (double *)(ey + (size_t)BI * ny);
    float2 *tall = (float2 *)tbuf.p;
    const float2 **ptab = (const float2 **)pbuf.p;
    const int last = checkpoints[ncheck - 1];
    const double dscale = (double)n2 * (double)n2;
    std::vector<const float2 *> hptab((size_t)nslice * BI);
    std::vector<double> hf(2 * (size_t)BI);
    PhononBuilder pb(c, at, fparams, g, nslice, radius, o, nconfig, sigma, seed);
    if ((rc = pb.init())) return rc;
    if ((rc = err_reset(c))) return rc;
    for (int c0 = 0; c0 < nconfig; c0 += BC) {
        const int nc = std::min(BC, nconfig - c0);
        // this batch's configurations: displaced atoms -> potential -> transmission stack
        for (int j = 0; j < nc; ++j)
            if ((rc = pb.build(c0 + j, tall + slab / sizeof(float2) * j))) return rc;
        SliceTables st;
        if ((rc = build_slice_tables(c, g, o, 1, dz.data(), st))) return rc;
        float2 *twr = twiddles(c, ny), *twc = twiddles(c, nx);
        if (!twr || !twc) return fail(c, MSL_E_NOMEM, "twiddle table allocation failed");
        std::vector<double> hk(nx + ny + 2 * ndet);
        for (int i = 0; i < nx; ++i) hk[i] = (double)(i < nx / 2 ? i : i - nx) / g->ax;
        for (int i = 0; i < ny; ++i) hk[nx + i] = (double)(i < ny / 2 ? i : i - ny) / g->by;
        for (int d = 0; d < ndet; ++d) {
            hk[nx + ny + d] = det->k_in[d] * det->k_in[d];
            hk[nx + ny + ndet + d] = det->k_out[d] * det->k_out[d];
        }
        if ((rc = upload(c, c->fxy, hk.data(), sizeof(double) * hk.size()))) return rc;
        const double *kxd = (const double *)c->fxy.p, *kyd = kxd + nx;
        CUDA_TRY(c, c->apchi.ensure(sizeof(float2) * n2 + n2));
        float2 *apchi = (float2 *)c->apchi.p;
        uint8_t *mask = (uint8_t *)(apchi + n2);
        const double lam = msl_wavelength(o->kev);
        LAUNCH_TRY(c, timed(c, MSL_PROF_OTHER, [&] { return msl::launch_probe_table(nx, ny, kxd, kyd, pr->k_in * pr->k_in, pr->k_out * pr->k_out,
                                              lam, pr->df, pr->cs, 1.0 / ((double)nx * ny), apchi,
                                              c->stream, &c->launches); }));
        LAUNCH_TRY(c, timed(c, MSL_PROF_OTHER, [&] { return msl::launch_detector_mask(nx, ny, kxd, kyd, ndet, kyd + ny, kyd + ny + ndet, mask,
                                                c->stream, &c->launches); }));
        int ntile;
        {
            ColArgs probe_cfg = col_args(g, st, twc, 0, w, 1, msl::COL_LOAD | msl::COL_STORE, c->dflag);
            ntile = ny / msl::plan_col_c_launch(nx, probe_cfg);
        }
        CUDA_TRY(c, c->partial.ensure(sizeof(double) * (size_t)ncheck * BI * ntile * ndet));
        double *partial = (double *)c->partial.p;
        for (int p0 = 0; p0 < nprobe; p0 += BP) {
            const int np_ = std::min(BP, nprobe - p0), nb = nc * np_;
            // image b = j * np_ + p: configuration c0 + j, probe p0 + p
            for (int j = 0; j < nc; ++j)
                for (int p = 0; p < np_; ++p) {
                    const int b = j * np_ + p;
                    hf[2 * b] = probe_xy[2 * (p0 + p)] / g->ax;
                    hf[2 * b + 1] = probe_xy[2 * (p0 + p) + 1] / g->by;
                    for (int s = 0; s < nslice; ++s)
                        hptab[(size_t)s * nb + b] = tall + slab / sizeof(float2) * j + n2 * s;
                }
            // the stream is idle here (synchronized after the previous block), so the
            // host tables can be reused
            CUDA_TRY(c, cudaMemcpyAsync(fxy, hf.data(), sizeof(double) * 2 * nb, cudaMemcpyHostToDevice, c->stream));
            CUDA_TRY(c, cudaMemcpyAsync(ptab, hptab.data(), sizeof(float2 *) * (size_t)nslice * nb,
                                        cudaMemcpyHostToDevice, c->stream));
            LAUNCH_TRY(c, timed(c, MSL_PROF_OTHER, [&] { return msl::launch_probe_shifts(nx, ny, nb, fxy, ex, ey, c->stream, &c->launches); }));
            ColArgs pa = col_args(g, st, twc, 0, w, nb, msl::COL_PROBE | msl::COL_INV | msl::COL_STORE, c->dflag);
            pa.apchi = apchi;
            pa.ex = ex;
            pa.ey = ey;
            LAUNCH_TRY(c, timed(c, MSL_PROF_COL, [&] { return msl::launch_col_pass(nx, pa, c->stream, c->nsm, &c->launches); }));
            int ic = 0;
            for (int s = 0; s <= last; ++s) {
                RowArgs r = row_args(g, twr, nullptr, w, nb, msl::ROW_LOAD | msl::ROW_INV | msl::ROW_TRANS | msl::ROW_FWD, c->dflag);
                r.trans_b = ptab + (size_t)s * nb;
                LAUNCH_TRY(c, timed(c, MSL_PROF_ROW, [&] { return msl::launch_row_pass(ny, r, c->stream, c->nsm, &c->launches); }));
                const bool detect = checkpoints[ic] == s;
                int cf = msl::COL_LOAD | msl::COL_FWD | msl::COL_PROP;
                if (detect) cf |= msl::COL_DETECT;
                if (s < last) cf |= msl::COL_INV | msl::COL_STORE;
                ColArgs ca = col_args(g, st, twc, 0, w, nb, cf, c->dflag);
                ca.detmask = mask;
                ca.ndet = ndet;
                ca.partial = partial + (size_t)ic * BI * ntile * ndet;
                LAUNCH_TRY(c, timed(c, MSL_PROF_COL, [&] { return msl::launch_col_pass(nx, ca, c->stream, c->nsm, &c->launches); }));
                if (detect) {
                    // += each configuration's sums in configuration order: the result
                    // does not depend on how configurations or probes were batched
                    LAUNCH_TRY(c, timed(c, MSL_PROF_OTHER, [&] { return msl::launch_detector_accumulate(
                                      nc, np_, ntile, ndet, ca.partial, dscale,
                                      od + ((size_t)p0 * ncheck + ic) * ndet, ncheck * ndet, c->stream,
                                      &c->launches); }));
                    ++ic;
                }
            }
            CUDA_TRY(c, cudaStreamSynchronize(c->stream));
            collect_profile(c);
            if ((rc = err_check(c))) return rc;
        }
    }
    if (!odev) CUDA_TRY(c, cudaMemcpyAsync(det_out, od, obytes, cudaMemcpyDeviceToHost, c->stream));
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    return MSL_OK;
}

}  // extern "C"
