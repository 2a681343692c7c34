// Internal host-side interface between the C ABI (msl_api.cu) and the kernels.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <mutex>
#include <vector>

#include "../../include/msl.h"

namespace msl {

// Launch set-up of one kernel, kept per device: cudaFuncSetAttribute acts on
// the current device only, so the dynamic shared-memory limit is raised and
// the occupancy computed once for every device that launches the kernel, and
// a mutex makes first launches from several host threads safe.
constexpr int kMaxDevices = 64;
struct KernelSetup {
    std::mutex mu;
    int per_sm[kMaxDevices] = {};
    // *out = resident CTAs per SM (at least 1; need_one: fail instead when none fit)
    template <class K> cudaError_t get(K kern, int threads, size_t smem, bool need_one, int *out) {
        int dev = 0;
        cudaError_t e = cudaGetDevice(&dev);
        if (e != cudaSuccess) return e;
        if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
        std::lock_guard<std::mutex> lock(mu);
        if (!per_sm[dev]) {
            e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            if (e != cudaSuccess) return e;
            int b = 0;
            e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, kern, threads, smem);
            if (e != cudaSuccess) return e;
            if (b < 1) {
                if (need_one) return cudaErrorInvalidConfiguration;
                b = 1;
            }
            per_sm[dev] = b;
        }
        *out = per_sm[dev];
        return cudaSuccess;
    }
};

// Every grid side the line transforms are built for.
#define MSL_FOR_EACH_SIDE(X) X(64) X(128) X(256) X(384) X(512) X(768) X(1024) X(2048)

// Row pass: contiguous lines of length ny (one line = one ix of one image).
enum RowFlags {
    ROW_LOAD = 1,    // load the line from `in` (else start from constant 1 + 0i)
    ROW_GENT = 2,    // start from exp(i * phase_scale * vpot) (FP64 phase)
    ROW_INV = 4,     // exp(-i) line transform
    ROW_TRANS = 8,   // multiply by trans[ix][iy]
    ROW_FWD = 16,    // exp(+i) line transform
    ROW_ACCUM = 32,  // accum[line][iy] += accum_w * |psi|^2 (FP64)
    ROW_NOSTORE = 64 // do not write the wave back
};

struct RowArgs {
    const float2 *in;
    float2 *out;        // may equal in
    int nlines;         // images * nx
    int nx;             // lines per image
    const float2 *trans;   // [nx][ny] of the current layer (ROW_TRANS)
    const float *vpot;     // [nx][ny] per image (ROW_GENT)
    double phase_scale;    // rad per unit of vpot (ROW_GENT)
    const float2 *tw;      // twiddle tables of the ny plan
    int flags;
    float scale;           // multiplies the output when != 1
    int *err;              // set to 1 when a bounded wait gives up (may be null)
    double *accum;         // [nlines][ny] (ROW_ACCUM)
    double accum_w;
    const float2 *const *trans_b;  // per-image transmission rows (replaces trans when set)
};

// Column pass: strided lines of length nx (one line = one iy of one image).
enum ColFlags {
    COL_LOAD = 1,     // load from `in`
    COL_PROBE = 2,    // start from apchi[ix][iy] * ex[b][ix] * ey[b][iy]
    COL_FWD = 4,      // exp(+i) line transform
    COL_PROP = 8,     // * py[iy] * px[ix] inside the band limit, 0 outside
    COL_DETECT = 16,  // annular detector partial sums of |psi|^2
    COL_INV = 32,     // exp(-i) line transform
    COL_STORE = 64,   // store to `out`
    COL_CTF = 128,    // * ctf[ix][iy] (objective lens transfer, full 2D table)
};

struct ColArgs {
    const float2 *in;
    float2 *out;
    int batch;        // images
    int ny;           // columns per image
    const float2 *tw; // twiddle tables of the nx plan
    int flags;
    const float2 *px, *py;    // propagator tables (py carries the 1/(nx ny) scale)
    const float *kx2, *ky2;   // float k^2 tables (freqn semantics)
    float k2max;
    const float2 *apchi;      // [nx][ny]
    const float2 *ex, *ey;    // [batch][nx], [batch][ny]
    const uint8_t *detmask;   // [nx][ny], bit d = detector d
    int ndet;
    double *partial;          // [batch][ny / C][ndet]
    int *err;                 // set to 1 when a bounded wait gives up (may be null)
    const float2 *ctf;        // [nx][ny] (COL_CTF)
    // per-image tables (replace px/py, kx2/ky2, k2max when set): prop_b[b] -> px[nx] py[ny],
    // k2_b[b] -> kx2[nx] ky2[ny], k2max_b[b]
    const float2 *const *prop_b;
    const float *const *k2_b;
    const float *k2max_b;
};

struct PotArgs {
    // atom position as its nearest pixel (ic, jc) plus the residue x - ic dxp,
    // y - jc dyp formed in FP64 and rounded to float (an atom on a pixel keeps
    // the FP64 residue there: r is then clamped to 1e-10 A as in vzatom)
    const int *ic, *jc;
    const float *fx, *fy;
    const float *xf, *yf;     // wrapped into [0, ax), [0, by), rounded to float (tile culling)
    const int *Z;
    const int *off;           // [nslice + 1] atom ranges per slice
    int nslice, nx, ny;
    double ax, by, dxp, dyp;
    float dxpf, dypf;         // pixel sizes rounded to float
    float rad2;               // radius^2 (float compare, r < radius)
    const float *sp;          // [104][12] A1 B1 A2 B2 A3 B3 C1 D1 C2 D2 C3 D3
    float *v;                 // [nslice][nx][ny]
    // tabulated radial profiles (nsp > 0): cubic pieces over [tab_r0, cutoff] per
    // species slot zslot[Z]; below tab_r0 the analytic form
    const float4 *tab;
    const int *zslot;
    int nsp;
    float tab_r0, tab_inv_h, tab_off;  // piece coordinate u = r tab_inv_h + tab_off (= (r - r0) / h)
};
constexpr int kPotTabN = 512;   // cubic pieces per species
constexpr int kPotMaxSp = 8;    // species the tabulated kernel takes (more: analytic kernel)
// Cubic pieces of vzatom (FP64) for the species zlist[nsp] over [r0, rmax]: [nsp][kPotTabN].
void potential_tables(const double *fparams, const int *zlist, int nsp, double r0, double rmax, float4 *out);

bool plan_supported(int n);
// Kernel families of a side's passes (the autotuner's choices), per device.
// FAM_TC: line DFTs as split-bf16 contractions on the tensor cores (msl_tcfft.cu;
// sides 256 and 512, the slice loop's passes; other passes of the side keep FAM_FAST);
// chosen by hand, not by the autotuner (it changes the arithmetic, not only the speed).
enum PassFamily { FAM_FAST = 0, FAM_TMA = 1, FAM_REG = 2, FAM_COUNT = 3, FAM_TC = 3 };
bool set_schedule(int n, int row_family, int col_family);
bool get_schedule(int n, int *row_family, int *col_family);
// Entries the twiddle buffer of side n needs (0: the plan's own tables only) and
// the tables appended for the two-stage row kernels, written into `tables`
// (which holds at least that many entries).
int row_two_twiddles_size(int n);
void append_row_two_twiddles(int n, float2 *tables);
// Columns per detector-partial tile of the slice loop's column pass for this
// call's buffers: 4 for the two-stage kernels (512, 1024), the TMA-fed
// kernel's tile width where the wave buffer allows TMA, else the register-only
// kernel's.
int plan_col_c(int n);
int plan_col_c_launch(int n, const ColArgs &a);
// Per-stage twiddle tables for side n (exp(+2 pi i r k / (NS R)) at [r][k]).
void plan_twiddles(int n, std::vector<float2> &out);
// The same tables written into out[cap]; returns the entry count, or -1 when
// the side is not built or cap is too small (nothing is allocated).
int plan_twiddles_into(int n, float2 *out, int cap);

// Host-side slice tables shared by every entry point (no allocation):
// spatial frequencies in float as freqn() (slicelib.cpp:433-463), the squared
// band limit in float (mulslice.cpp:481-489), and the propagator tables of one
// thickness (mulslice.cpp:494-513), py carrying the ifft scale 1/(nx ny).
void freqn_f32(int n, double a, float *k, float *k2);
float k2max_f32(int nx, int ny, double ax, double by, double bw);
void prop_tables(int nx, int ny, const msl_optics *o, double dz, const float *kx, const float *kx2,
                 const float *ky, const float *ky2, float2 *px, float2 *py);

// Each launcher returns cudaSuccess or the launch error; *launches is bumped.
cudaError_t launch_row_pass(int ny, const RowArgs &a, cudaStream_t s, int nsm, int64_t *launches);
cudaError_t launch_col_pass(int nx, const ColArgs &a, cudaStream_t s, int nsm, int64_t *launches);
cudaError_t launch_potential(const PotArgs &a, cudaStream_t s, int64_t *launches);
// apchi[ix][iy] = A(s) exp(-i chi(s)) * scale, s = kx^2 + ky^2 from kxd/kyd (FP64)
cudaError_t launch_probe_table(int nx, int ny, const double *kxd, const double *kyd, double s_in,
                               double s_out, double lam, double df, double cs, double scale,
                               float2 *apchi, cudaStream_t s, int64_t *launches);
// ex[b][ix] = exp(2 pi i * sidx(ix) * fx[b]), same for ey
cudaError_t launch_probe_shifts(int nx, int ny, int nb, const double *fxy, float2 *ex, float2 *ey,
                                cudaStream_t s, int64_t *launches);
// bit d of mask[ix][iy] set when kin2[d] <= s <= kout2[d]
cudaError_t launch_detector_mask(int nx, int ny, const double *kxd, const double *kyd, int ndet,
                                 const double *kin2, const double *kout2, uint8_t *mask,
                                 cudaStream_t s, int64_t *launches);
// ctf[ix][iy] = exp(-i chi(k)) * scale for k2 = kx2 + ky2 (float) <= k2obj, else 0;
// chi = pi lam k2 (cs lam^2 k2 / 2 - df) in FP64
struct CtfParams {
    double lam, cs, df, dfa2, dfa2phi, dfa3, dfa3phi;
    float k2obj, scale;
};
// phi = atan2(ky, kx) from the float kx / ky tables (astigmatism terms)
cudaError_t launch_ctf_table(int nx, int ny, const float *kx2, const float *ky2, const float *kx,
                             const float *ky, const CtfParams &p, float2 *ctf, cudaStream_t s,
                             int64_t *launches);
// out[b][ix][iy] = exp(2 pi i (qx[b] xpos[ix] + qy[b] ypos[iy])), the sum in float as mulslice.cpp:573-577
cudaError_t launch_tilt_waves(int nx, int ny, int nb, const float *xpos, const float *ypos,
                              const float *q, float2 *out, cudaStream_t s, int64_t *launches);
// a kernel whose mbarrier wait must run out: raises *err
cudaError_t launch_wait_timeout(int *err, uint32_t polls, cudaStream_t s, int64_t *launches);
// out[b * out_stride + d] = scale * sum_t partial[b][t][d]
cudaError_t launch_transmission_phase(const float *v, double scale, size_t n, float2 *t, int nsm, cudaStream_t s,
                                      int64_t *launches);
// out[p * out_stride + d] += scale * sum_t partial[j * np + p][t][d] for j = 0..nconf-1 in order
cudaError_t launch_detector_accumulate(int nconf, int np, int ntile, int ndet, const double *partial,
                                       double scale, double *out, int out_stride, cudaStream_t s,
                                       int64_t *launches);
// D[M][N] (FP32) = A[M][K] * B[N][K]^T, bf16 operands, on the tensor cores
// (tcgen05, accumulator in tensor memory); M % 128 == 0, K % 64 == 0,
// 16 <= N <= 256, N % 16 == 0.  *err is raised if an MMA completion wait gives up.
cudaError_t launch_tc_gemm(const void *A, const void *B, float *D, int M, int N, int K, int *err,
                           cudaStream_t s, int64_t *launches);
// ------------------------------------------------ tensor-core line DFTs (msl_tcfft.cu)
enum TcMode { TC_MODE_NONE = 0, TC_MODE_TRANS = 1, TC_MODE_PROP = 2 };
struct TcPassArgs {
    float2 *data;               // waves [images][nx][ny], in place
    int nlines;                 // rows: images * nx; columns: images * ny (multiple of 8)
    int nx, ny;
    int cols;                   // 0: row lines (along iy), 1: column lines (along ix)
    int dir1, dir2;             // signs of the first and second transform
    int second;                 // 0: stop after the pointwise step (detection only)
    int mode;                   // TcMode pointwise step between the transforms
    const float2 *trans;        // TC_MODE_TRANS: [nx][ny] of the layer
    const float2 *const *trans_b;  // or per-image pointers
    const float2 *px, *py;      // TC_MODE_PROP
    const float *kx2, *ky2;
    float k2max;
    const uint8_t *detmask;     // column passes: detector bits [nx][ny] (null: none)
    int ndet;
    double *partial;            // [images][ny / 8][ndet]
    int *err;
};
bool tc_side(int n);
int tc_col_tile();
cudaError_t launch_tc_pass(const TcPassArgs &a, cudaStream_t s, int nsm, int64_t *launches);

// ------------------------------------------ on-chip STEM slice loop (msl_resident.cu)
// One 8-CTA cluster per probe, the 256^2 wave resident in the cluster's shared
// memory across slices.  All pointers are device pointers.
struct ResidentArgs {
    const float2 *w0;          // [nprobe][256][256] entrance waves (after the probe's x inverse)
    const float2 *trans;       // [ntrans][256][256]
    const float2 *prop;        // [ntrans][px 256 | py 256]
    const float *kx2, *ky2;    // float k^2 tables
    float k2max;
    const uint8_t *mask;       // [256][256] detector bits
    int ndet;
    const int *layer_seq;      // [nslice]
    int nslice;
    const int *checkpoints;    // [ncheck] ascending slice indices
    int ncheck;
    double *partial;           // [ncheck][nprobe][8][ndet]
    int nprobe;
    int *err;                  // raised when a bounded wait for a peer's copies gives up
};
cudaError_t launch_stem_resident(const ResidentArgs &a, cudaStream_t s, int nsm, int64_t *launches);
int resident_side();
int resident_cluster();

// ------------------------------------------------- learned closure (msl_closure.cu)
// The network's parameters, Adam state and work buffers on one device.
struct ClosureNet {
    float *params = nullptr, *grads = nullptr, *adam_m = nullptr, *adam_v = nullptr;
    __nv_bfloat16 *wt = nullptr;      // expanded bf16 weights of the tensor-core layers
    float *dwreal = nullptr;          // one layer's real weight gradient + bias gradient
    void *acts = nullptr;             // activations
    float *partial = nullptr;         // weight-gradient partial sums
    double *loss_part = nullptr;      // per-block loss sums
    float *scale = nullptr;           // per-image s and 1/s
    size_t cap_pix = 0;
    int cap_img = 0;
    bool cap_train = false;
    int step = 0;
    int loss_blocks = 0;
    __nv_bfloat16 *hbuf[6] = {}, *dh[2] = {}, *xbuf = nullptr;
    float *g6 = nullptr;
    cudaError_t alloc_params();
    void release();
    cudaError_t ensure(size_t npix, int nimg, bool train);
    cudaError_t expand(cudaStream_t s, int nsm, int64_t *launches);
    cudaError_t conv_tc(const __nv_bfloat16 *in, const __nv_bfloat16 *w, const float *bias,
                        const __nv_bfloat16 *mask, __nv_bfloat16 *out, int B, int H, int W, int epi, int *err,
                        cudaStream_t s, int nsm, int64_t *launches);
    cudaError_t forward(const float2 *psi, int B, int H, int W, float2 *out, const float2 *target, bool train,
                        int *err, cudaStream_t s, int nsm, int64_t *launches);
    cudaError_t backward(int B, int H, int W, int *err, cudaStream_t s, int nsm, int64_t *launches);
    cudaError_t adam(float lr, cudaStream_t s, int nsm, int64_t *launches);
};
int closure_param_count();
void closure_init_params(uint64_t seed, std::vector<float> &h);

cudaError_t launch_detector_finalize(int nb, int ntile, int ndet, const double *partial,
                                     double scale, double *out, int out_stride, cudaStream_t s,
                                     int64_t *launches);

}  // namespace msl
