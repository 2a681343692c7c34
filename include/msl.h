/*
 * msl.h — C ABI of the GB300 multislice library (libmsl.so).
 *
 * The library replaces the reference's hot path on one GPU:
 *   projected potential  ->  per-slice transmit / 2D FFT / Fresnel propagate /
 *   inverse FFT          ->  STEM annular detection.
 * Every entry point is a plain C function over plain pointers and sizes; no
 * CUDA or framework type appears in a signature.  Buffers are owned by the
 * caller and may live in host memory or in device memory of the context's GPU:
 * the library inspects each pointer (cudaPointerGetAttributes) and copies host
 * buffers in and out itself.  Calls are synchronous: when one returns, its
 * outputs are complete.  All calls return MSL_OK (0) or a negative MSL_E_*
 * status; msl_last_error() gives the message of the context's last failure.
 * One context per host thread; a context drives one GPU.
 *
 * Conventions (those of Kirkland's mulslice, ImageSimulation/multislice):
 *   - a wave or image of nx*ny complex64 values is x-major: element (ix, iy)
 *     sits at index iy + ix*ny (cfpix.hpp:99-125), stored as (re, im) floats;
 *   - "fft" is exp(+2 pi i ...) and unscaled, "ifft" is exp(-2 pi i ...) and
 *     scaled by 1/(nx*ny) (cfpix.cpp:115-230, FFTW_BACKWARD / FFTW_FORWARD);
 *   - spatial frequency of index i is i/a for i <= (n/2 rounded), else (i-n)/a
 *     (slicelib.cpp:433-463);
 *   - lengths in Angstrom, energies in keV, angles in radians, potentials in
 *     volt-Angstrom.
 * Supported grid sides: 64, 128, 256, 384, 512, 768, 1024, 2048 (nx and ny
 * chosen independently).
 */
#ifndef MSL_H
#define MSL_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MSL_OK 0
#define MSL_E_ARG (-1)        /* invalid argument (size, range, NaN, null)   */
#define MSL_E_CUDA (-2)       /* a CUDA runtime call failed                  */
#define MSL_E_NOMEM (-3)      /* device or host allocation failed            */
#define MSL_E_UNSUPPORTED (-4) /* grid side or option not built              */

#define MSL_MAX_DETECTORS 8

typedef struct msl_ctx msl_ctx;

/* Cell and sampling: nx x ny pixels over ax x by Angstrom. */
typedef struct {
    int nx, ny;
    double ax, by;
} msl_grid;

/* Atom list (the .coo content after conversion to Cartesian Angstrom,
 * amodel/include/ModelCoo.cpp:20-90).  z runs along the beam; cz is the
 * specimen thickness that is cut into slices. */
typedef struct {
    int natom;
    const double *x, *y, *z; /* Angstrom */
    const int *Z;            /* atomic numbers 1..103 */
    double cz;               /* thickness, Angstrom */
} msl_atoms;

/* Electron optics of the slice loop. */
typedef struct {
    double kev;          /* beam energy */
    double bandlimit;    /* fraction of the Nyquist radius kept; 2/3 in mulslice.cpp:24 */
    double tilt_x, tilt_y; /* crystal tilt (rad), mulslice.cpp:497-513 */
    int f32_prop_args;   /* 0: propagator arguments in FP64 (default);
                            1: built in float exactly as mulslice.cpp:499-513 */
} msl_optics;

/* Converged STEM probe (MSProject.cs:458-514), reciprocal lengths in 1/A. */
typedef struct {
    double k_in, k_out;  /* aperture: k_in^2 <= |k|^2 <= k_out^2 */
    double df;           /* defocus, Angstrom */
    double cs;           /* spherical aberration, Angstrom */
} msl_probe;

/* Annular detectors (MSProject.cs:792-842): detector d sums |Psi(k)|^2 over
 * k_in[d]^2 <= |k|^2 <= k_out[d]^2 (1/A), bounds inclusive. */
typedef struct {
    int ndet;
    const double *k_in, *k_out;
} msl_detectors;

/* ---------------------------------------------------------------- context */

/* Create a context on CUDA device `device`.  Allocates the context's stream
 * and lazily its work buffers.  Replaces the device set-up of
 * LMultiSlice/Dispatcher.cu:191-207. */
int msl_ctx_create(int device, msl_ctx **out);
int msl_ctx_destroy(msl_ctx *ctx);
/* Message of the last failed call on ctx (static string owned by ctx). */
const char *msl_last_error(const msl_ctx *ctx);
/* Library version string. */
const char *msl_version(void);
/* Number of kernels this context has launched since creation. */
int64_t msl_kernel_launches(const msl_ctx *ctx);

/* ------------------------------------------------------------ parameters */

/* Parse FPARAMS.DAT text (ImageSimulation/parserFPARAMS/FPARAMS.DAT; reader
 * parserFPARAMS/main.cpp:18-98) into tab[104*12]: row Z holds
 * a1 b1 a2 b2 a3 b3 c1 d1 c2 d2 c3 d3, row 0 is zero. */
int msl_fparams_parse(const char *text, size_t len, double *tab);

/* Unit cell and atom records of a .coo file. */
typedef struct {
    double a, b, c;            /* cell edges, Angstrom */
    double alpha, beta, gamma; /* cell angles, degrees */
    int natom;
} msl_cell;

/* Parse .coo text: a header "a b c alpha beta gamma natoms" then one line per
 * atom "x y z Z [dw] [ads] [occ]" in fractional coordinates, wrapped into
 * [0, 1); blank lines are skipped and "//" starts a comment (the C# reader,
 * MSProject.cs:239-338); a first line that is not a header is taken as a title
 * (the amodel reader, amodel/include/ModelCoo.cpp:20-90).  Missing dw, ads
 * default to 0 and occ to 1.  rec receives natom records of 7 doubles
 * (x y z Z dw ads occ) when it is not NULL and capacity >= natom; call with
 * rec = NULL first to learn natom from cell->natom. */
int msl_coo_parse(const char *text, size_t len, msl_cell *cell, double *rec, int capacity);

/* Electron wavelength (A) and interaction constant sigma (rad/(kV*A)):
 * slicelib.cpp:2795-2806 and :2387-2412. */
double msl_wavelength(double kev);
double msl_sigma(double kev);

/* ------------------------------------------------------------- potential */

/* Projected potential V_z of every slice: the PotentialBuilder step.
 * Replaces ModelPotential::calculatePotentialGrid (LMultiSlice/ModelPotential.cu:27-99,
 * kernel :125-230, atom form :232-292) with Kirkland's vzatom form
 * (slicelib.cpp:2666-2716) and FPARAMS coefficients `fparams[104*12]`.
 * Atoms are binned by floor(z / (cz/nslice)); those outside [0, cz) are
 * dropped.  Each pixel sums, over the atoms of its slice, vzatom(Z, r) for the
 * single minimum image with r < radius (r clamped below at 1e-10 A);
 * radius must be below half of ax and of by.
 * v_out: float [nslice][nx][ny] (host or device). */
int msl_potential_build(msl_ctx *ctx, const msl_atoms *atoms, const double *fparams,
                        const msl_grid *grid, int nslice, double radius, float *v_out);

/* Band-limited transmission functions t = exp(i sigma V_z) of nlayer slices:
 * mulslice.cpp:414-421 (phase), :515-522 (fft -> zero |k| beyond the band
 * limit -> ifft).  The phase sigma*V is formed in FP64 before exponentiation.
 * v: float [nlayer][nx][ny]; t_out: complex64 [nlayer][nx][ny]. */
int msl_transmission_build(msl_ctx *ctx, const msl_grid *grid, const msl_optics *optics,
                           const float *v, int nlayer, float *t_out);

/* -------------------------------------------------------------- the FFT */

/* In-place 2D transform of `batch` complex64 images, Kirkland's cfpix::fft
 * (dir = +1: exp(+i), unscaled) or cfpix::ifft (dir = -1: exp(-i), x 1/(nx*ny))
 * (cfpix.cpp:115-167). */
int msl_fft2d(msl_ctx *ctx, const msl_grid *grid, float *psi, int batch, int dir);

/* ------------------------------------------------------------ multislice */

/* Coherent multislice of a batch of waves: for islice in 0..nslice-1 with
 * l = layer_seq[islice]: psi *= trans[l]; fft; propagate with the separable
 * Fresnel propagator of thickness dz[l] and the band limit; ifft
 * (mulslice.cpp:706-739, propagate slicelib.cpp:744-790).  Replaces
 * ModelSimulated::imageCalculation's slice loop (ModelSimulated.cu:52-119).
 * trans: complex64 [ntrans][nx][ny]; dz: double [ntrans];
 * psi: complex64 [batch][nx][ny], in: entrance waves, out: exit waves;
 * psi == NULL is not allowed; to start from a plane wave of amplitude 1 pass
 * plane_wave = 1 (psi is then output only). */
int msl_multislice(msl_ctx *ctx, const msl_grid *grid, const msl_optics *optics,
                   const float *trans, int ntrans, const double *dz,
                   const int *layer_seq, int nslice, float *psi, int batch, int plane_wave);

/* STEM scan and detect: for each probe position (x, y) in probe_xy[nprobe*2]
 * build the converged probe (MSProject.cs:458-514), run the slice loop, and
 * after the propagator of every slice listed in checkpoints[ncheck]
 * (ascending, 0-based; MSReuseCalculator.cs:36-92) sum |Psi(k)|^2 over each
 * annulus (MSProject.cs:792-842).  Sums are FP64 and in the reference's scale
 * (unscaled forward transform of a wave whose reciprocal-space probe has unit
 * amplitude inside the aperture).  det_out: double [nprobe][ncheck][ndet]. */
int msl_stem_scan(msl_ctx *ctx, const msl_grid *grid, const msl_optics *optics,
                  const float *trans, int ntrans, const double *dz, const int *layer_seq,
                  int nslice, const msl_probe *probe, const double *probe_xy, int nprobe,
                  const msl_detectors *det, const int *checkpoints, int ncheck,
                  double *det_out);

/* Per-kernel timing.  When enabled, every launch of the context is bracketed
 * by CUDA events on the context's stream and its duration is added to the
 * totals of its kind (row pass, column pass, potential, other).  Enabling
 * resets the totals.  The reference times its phases the same way
 * (ModelPotential.cu:46-50,92-96; ModelSimulated.cu:43-47,178-182). */
#define MSL_PROF_ROW 0
#define MSL_PROF_COL 1
#define MSL_PROF_POTENTIAL 2
#define MSL_PROF_OTHER 3
#define MSL_PROF_KINDS 4
int msl_profile_enable(msl_ctx *ctx, int on);
int msl_profile_read(const msl_ctx *ctx, int kind, int64_t *launches, double *ms);

/* ------------------------------------------------------- CTEM imaging */

/* Objective lens of the CTEM image (mulslice.cpp:539-676): the exit wave's
 * spectrum is multiplied by exp(-i chi(k)) inside the objective aperture
 * k^2 <= k_obj^2, chi = pi lambda k^2 (Cs lambda^2 k^2 / 2 - df
 * + dfa2 sin(2(phi - dfa2phi)) + (2/3) dfa3 lambda |k| sin(3(phi - dfa3phi))),
 * phi = atan2(ky, kx) (mulslice.cpp:613-619), and |ifft|^2 is summed over defocus
 * values df + j*df_step, |j| <= 2.5 df_spread / df_step, with Gaussian weights
 * exp(-(j df_step / df_spread)^2 / 2) normalised to 1 (df_spread = 0: one
 * coherent image).  chi is evaluated in FP64. */
typedef struct {
    double cs;         /* spherical aberration, Angstrom */
    double df;         /* mean defocus, Angstrom (Kirkland's sign) */
    double k_obj;      /* objective aperture radius, 1/A */
    double df_spread;  /* defocus spread (standard deviation), Angstrom; 0 = none */
    double df_step;    /* defocus integration step, Angstrom (used when df_spread > 0) */
    double dfa2, dfa2phi; /* 2-fold astigmatism: magnitude (A), angle (rad) */
    double dfa3, dfa3phi; /* 3-fold astigmatism: magnitude (A), angle (rad) */
} msl_lens;

/* CTEM image of a batch of waves: runs the slice loop of msl_multislice on psi
 * (plane_wave = 1: start from amplitude 1), then images every exit wave through
 * the lens and adds weight * sum over the batch of the (defocus-averaged) image
 * intensity into image[nx][ny] (FP64, accumulated, not cleared).  psi receives
 * the exit waves.  When exit_intensity is not NULL, weight * |exit wave|^2 is
 * added to it the same way. */
int msl_ctem_image(msl_ctx *ctx, const msl_grid *grid, const msl_optics *optics,
                   const float *trans, int ntrans, const double *dz, const int *layer_seq,
                   int nslice, const msl_lens *lens, float *psi, int batch, int plane_wave,
                   double weight, double *image, double *exit_intensity);

/* Kirkland's partial-coherence CTEM image (mulslice.cpp:539-676): the plane
 * wave is tilted to every illumination angle (qx, qy) = (i/ax, j/by) with
 * acmin <= lambda |q| <= acmax (radians), each tilted wave runs the slice loop
 * (all angles in one batch), is imaged through the lens with the defocus
 * spread, and image[nx][ny] (FP64, overwritten) receives the average over
 * angles and defocus values.  n_angles (may be NULL) returns the angle count. */
int msl_ctem_partial_coherence(msl_ctx *ctx, const msl_grid *grid, const msl_optics *optics,
                               const float *trans, int ntrans, const double *dz,
                               const int *layer_seq, int nslice, const msl_lens *lens,
                               double acmin, double acmax, double *image, int *n_angles);

/* Frozen-phonon displacements (MSUseOnceCalculator.cs:179-199 jitters every atom
 * by a Gaussian per axis; the reference's System.Random stream cannot be
 * reproduced, so this library defines its own): for configuration `config`,
 * atom i and axis a the displacement is sigma * n, n a standard normal from the
 * Box-Muller transform of two uniforms u = (splitmix64(key) >> 11) * 2^-53,
 * key = seed ^ splitmix64((config << 40) | (i << 2) | k), k = 0..3; axes x, y
 * use the cos and sin of the first pair, z the cos of the second.
 * d_out: double [natom][3]. */
int msl_phonon_displacements(uint64_t seed, int config, int natom, double sigma, double *d_out);

/* Amorphous specimen of the uneven-batch workload (host code): atoms uniform in
 * a bx x by x thickness box at `density` atoms / A^3 with no two closer than
 * dmin (periodic in x and y), thrown one by one from the library's splitmix64
 * stream of `seed` onto a grid of cells of side >= dmin and kept when no
 * accepted atom of the 27 neighbouring cells is too close; Z drawn from zs[nz]
 * with the given weights.  xyz[3 * count] (Angstrom) and Z[count] receive
 * round(density * volume) atoms (fewer only if 100 throws per atom cannot
 * place them); when capacity is too small the call returns MSL_E_ARG with the
 * needed count in *count.  No counterpart in the reference (its specimens come
 * from .coo files). */
int msl_amorphous(uint64_t seed, double bx, double by, double thickness, double density, double dmin, int nz,
                  const int *zs, const double *weights, int capacity, double *xyz, int *Z, int *count);

/* Frozen-phonon CTEM: for each of nconfig configurations displace the atoms
 * (msl_phonon_displacements), build the potential and transmission functions
 * of nslice equal slices, run a plane wave through them and image it; image and
 * exit_intensity (either may be NULL) receive the averages over configurations,
 * double [nx][ny] (overwritten).  Configurations run in batches through one
 * slice loop, as many as 16 GiB of transmission functions hold (half the
 * context's memory limit when one is set); the averages do not depend on the
 * batch size. */
int msl_frozen_phonon(msl_ctx *ctx, const msl_atoms *atoms, const double *fparams,
                      const msl_grid *grid, int nslice, double radius, const msl_optics *optics,
                      const msl_lens *lens, int nconfig, double sigma, uint64_t seed,
                      double *image, double *exit_intensity);

/* Frozen-phonon STEM (the thermal-vibration loop wrapped around every probe
 * position: MSProjectUseOnce.cs:235-273, jitter MSUseOnceCalculator.cs:179-199
 * with MusliRandom.Vobble, MusliRandom.cs:43-55).  For each of nconfig
 * configurations the atoms are displaced (msl_phonon_displacements with seed
 * and sigma), the potential and transmission functions of nslice equal slices
 * are built, and every probe of probe_xy runs the slice loop with detection at
 * the checkpoints as msl_stem_scan does.  det_out[nprobe][ncheck][ndet]
 * receives the detector sums added over the configurations, as the reference
 * adds each configuration into its STEM image (MSProject.cs:836-837; divide
 * by nconfig for the average).  Configurations x probes run together as one
 * batch of waves through one slice loop, each wave reading its own
 * configuration's transmission rows; each probe's sums are added in
 * configuration order in FP64, so the result does not depend on the batch
 * sizes (msl_set_probe_batch, memory cap). */
int msl_stem_scan_phonon(msl_ctx *ctx, const msl_atoms *atoms, const double *fparams,
                         const msl_grid *grid, int nslice, double radius, const msl_optics *optics,
                         const msl_probe *probe, const double *probe_xy, int nprobe,
                         const msl_detectors *det, const int *checkpoints, int ncheck, int nconfig,
                         double sigma, uint64_t seed, double *det_out);

/* ------------------------------------------------------ tensor cores */

/* D[M][N] (FP32) = A[M][K] * B[N][K]^T with bf16 operands (raw 16-bit
 * patterns, row-major) on the tensor cores (tcgen05.mma, accumulator in tensor
 * memory).  M % 128 == 0, K % 64 == 0, 16 <= N <= 256 and N % 16 == 0.  No
 * counterpart in the reference: the contraction under the learned
 * coarse-slice closure, exported so it can be checked on its own. */
int msl_tc_gemm_bf16(msl_ctx *ctx, const uint16_t *A, const uint16_t *B, float *D, int M, int N, int K);

/* ------------------------------------------- learned coarse-slice closure */

/* A small complex-valued convolutional network that corrects an exit wave
 * computed with 4x thicker slices toward the fine-slice result (no counterpart
 * in the reference; the reference's fine-slice loop, mulslice.cpp:706-739, is
 * its fallback and the judge of its error).  Six complex 3x3 convolutions with
 * periodic boundaries -- 1 -> 32 -> 32 -> 32 -> 32 -> 32 -> 1 channels, CReLU
 * between them -- act on the wave divided by s = sqrt(sum |psi|^2 / 256^2) (its
 * RMS on a 256^2 grid, so a probe keeps its per-pixel scale on any grid), and
 * the output adds s times the result to the wave.  Parameters are FP32 master copies used as
 * bf16; the 32 -> 32 layers run on the tensor cores (forward and input
 * gradient), the rest on the CUDA cores; training uses Adam.  Waves are
 * complex64 [batch][h][w] (w a multiple of 128, h >= 3), host or device. */
typedef struct msl_closure msl_closure;
int msl_closure_create(msl_ctx *ctx, uint64_t seed, msl_closure **out);
int msl_closure_destroy(msl_closure *net);
/* Number of FP32 parameters: per layer, weights [9][co][ci][2] then bias [co][2]. */
int msl_closure_param_count(void);
int msl_closure_get_params(msl_ctx *ctx, const msl_closure *net, float *params);
/* Replaces the parameters and resets the optimiser state. */
int msl_closure_set_params(msl_ctx *ctx, msl_closure *net, const float *params);
/* psi <- psi + s * net(psi / s), in place. */
int msl_closure_apply(msl_ctx *ctx, msl_closure *net, float *psi, int batch, int h, int w);
/* Loss L = mean over pixels of |net(coarse / s) - (fine - coarse) / s|^2 and
 * its gradient dL/dparams (grad may be NULL). */
int msl_closure_gradients(msl_ctx *ctx, msl_closure *net, const float *coarse, const float *fine, int batch,
                          int h, int w, float *grad, double *loss);
/* One Adam step (lr; beta 0.9 / 0.999) on that loss; *loss before the step. */
int msl_closure_train_step(msl_ctx *ctx, msl_closure *net, const float *coarse, const float *fine, int batch,
                           int h, int w, float lr, double *loss);

/* Exit waves of a STEM scan: each probe of probe_xy (msl_stem_scan's probe)
 * through the slice loop of msl_multislice; psi_out: complex64
 * [nprobe][nx][ny] in real space (host or device).  The probe-and-slice part
 * of MSProjectReuse.cs:254-347 without detection. */
int msl_stem_exit_waves(msl_ctx *ctx, const msl_grid *grid, const msl_optics *optics, const float *trans,
                        int ntrans, const double *dz, const int *layer_seq, int nslice, const msl_probe *probe,
                        const double *probe_xy, int nprobe, float *psi_out);

/* STEM scan through coarse slices corrected by the closure: every probe runs
 * the slice loop over (typically 4x thicker) layers, its real-space exit wave
 * is corrected by msl_closure_apply, and the corrected wave's spectrum inside
 * the band limit is summed over each annulus (msl_stem_scan's detector, in its
 * scale).  det_out: double [nprobe][ndet].  ny must be a multiple of 128. */
int msl_stem_scan_closure(msl_ctx *ctx, msl_closure *net, const msl_grid *grid, const msl_optics *optics,
                          const float *trans, int ntrans, const double *dz, const int *layer_seq, int nslice,
                          const msl_probe *probe, const double *probe_xy, int nprobe, const msl_detectors *det,
                          double *det_out);

/* msl_stem_scan with every probe's wave kept on chip across all slices
 * (arguments, outputs and conventions as msl_stem_scan): one 8-CTA thread-block
 * cluster per probe holds the 256 x 256 wave in its shared memory (32 rows per
 * CTA); row transforms run in place, column transforms gather and scatter
 * through distributed shared memory, so HBM sees the probe once and the
 * transmission rows, not the wave every slice.  Built for 256^2 grids (the
 * 512^2 wave and its exchange space exceed a 16-CTA cluster's shared memory);
 * other sides return MSL_E_UNSUPPORTED.  The reference's scan is serial over
 * probes (MSProjectReuse.cs:254-347). */
int msl_stem_scan_resident(msl_ctx *ctx, const msl_grid *grid, const msl_optics *optics, const float *trans,
                           int ntrans, const double *dz, const int *layer_seq, int nslice, const msl_probe *probe,
                           const double *probe_xy, int nprobe, const msl_detectors *det, const int *checkpoints,
                           int ncheck, double *det_out);

/* ------------------------------------------------------- uneven batches */

#define MSL_PLANE_WAVE 0
#define MSL_PROBE 1

/* One multislice job of an uneven batch: its own grid, energy, transmission
 * stack, slice sequence and illumination (a plane wave of amplitude 1, or the
 * converged probe of MSProject.cs:458-514 at (probe_x, probe_y)). */
typedef struct {
    msl_grid grid;
    double kev;
    const float *trans;      /* complex64 [ntrans][nx][ny], host or device */
    int ntrans;
    const double *dz;        /* [ntrans] slice thicknesses */
    const int *layer_seq;    /* [nslice] */
    int nslice;
    int illumination;        /* MSL_PLANE_WAVE or MSL_PROBE */
    msl_probe probe;
    double probe_x, probe_y; /* Angstrom */
    float *exit_wave;        /* out: complex64 [nx][ny], host or device */
} msl_job;

/* Run many independent slice loops at once (the reference runs them one after
 * another: MSProjectReuse.cs:254-347, MSProjectUseOnce.cs:235-273).  Jobs are
 * grouped by grid shape; inside a group every slice step is one row-pass and
 * one column-pass launch over all jobs still running (jobs ordered by
 * decreasing slice count, so the running ones form a prefix), each image with
 * its own transmission rows, propagator and band-limit tables.  Results equal
 * msl_multislice run job by job.  bandlimit as in msl_optics. */
int msl_run_jobs(msl_ctx *ctx, const msl_job *jobs, int njobs, double bandlimit);

/* Check of the failure path of the library's bounded waits: launches a kernel
 * whose mbarrier wait (polled `polls` times) nothing ever completes.  Returns
 * MSL_OK when the wait gave up and the kernel raised the context's error flag
 * as designed -- no fault, no hang, the context stays usable -- and MSL_E_CUDA
 * otherwise.  Every TMA wait in the pass kernels takes the same path. */
int msl_check_wait_timeout(msl_ctx *ctx, uint32_t polls);

/* Pass schedules and their autotuner.  Each grid side's row and column passes
 * can run on one of three kernel families: MSL_FAM_FAST (warp-owned, two-stage
 * and warp-pair line kernels fed by bulk / TMA copies; the default),
 * MSL_FAM_TMA (TMA-tiled kernels with block-wide exchanges) or MSL_FAM_REG
 * (register-only kernels with plain loads).  All compute the same transforms
 * (not bit for bit: their radix plans differ).  msl_autotune times one slice
 * step of `batch` synthetic waves of `side` for every pair of families (`reps`
 * steps each after a warm-up, CUDA events on the context's stream), keeps the
 * fastest pair as the schedule of that side on the context's device, and
 * returns it and the times (ms[row_family * 3 + col_family], ms per step; may
 * be NULL).  With msl_set_autotune(ctx, 1), msl_multislice and msl_stem_scan
 * tune each side once per device on first use (waves of 256 MiB).  The
 * reference has no counterpart (cuFFTW plans its own transforms). */
#define MSL_FAM_FAST 0
#define MSL_FAM_TMA 1
#define MSL_FAM_REG 2
/* The tensor-core form of the slice loop's passes (sides 256 and 512): every
 * line DFT as two dense contractions (four-step, 16 x N/16) on tcgen05 with
 * split-bf16 products (hi + lo per operand, three products, FP32 accumulate),
 * twiddles, transmission, propagator and detector sums as in the FP32 passes.
 * Set with msl_set_schedule only (the autotuner times the FP32 families); the
 * other passes of the side (probe formation, the plane-wave first slice, the
 * closing inverse) keep MSL_FAM_FAST. */
#define MSL_FAM_TC 3
int msl_autotune(msl_ctx *ctx, int side, int batch, int reps, int *row_family, int *col_family, double *ms);
int msl_set_schedule(msl_ctx *ctx, int side, int row_family, int col_family);
int msl_get_schedule(msl_ctx *ctx, int side, int *row_family, int *col_family);
int msl_set_autotune(msl_ctx *ctx, int on);

/* Probe batch size used by msl_stem_scan (0 = automatic).  Work buffers are
 * sized batch * nx * ny * 8 bytes. */
int msl_set_probe_batch(msl_ctx *ctx, int batch);

/* Cap on the device memory the context keeps in its work buffers (0 = none,
 * the default), for GPUs shared with other work.  A call whose buffers would
 * grow past the cap returns MSL_E_NOMEM before it frees or allocates anything
 * and leaves the context usable; the automatic probe batch of msl_stem_scan
 * shrinks to half the cap.  Caller-owned buffers are not counted.  The
 * reference has no counterpart (its buffers are sized by the calculation). */
int msl_set_memory_limit(msl_ctx *ctx, size_t bytes);
/* Bytes the context's work buffers hold now. */
int msl_memory_in_use(msl_ctx *ctx, size_t *bytes);

/* ------------------------------------------------- Muslib-shaped exports */

/* The reference's native STEM library (Musli console 1.3 (STEM) 2/Muslib) with
 * identical argument lists, so its C# P/Invoke declarations bind unchanged
 * (Windows ULONG/LONG are 32-bit).  Host arrays in the C# layout: N x M complex
 * doubles, element (i, j) at gli[2*(j*N + i)].  Run on the current CUDA device
 * in FP64; return 0 (success) or -1.  *cpro advances as the reference's does
 * (periodic forms end at 100, clipped forms add 100/Na per atom).
 * CreatePropagator / ApplyPropagator: Propagator.cpp:5-53 / :55-107. */
int CreatePropagator(double a, double b, double gam, double thickness, double E, double Xtilt,
                     double Ytilt, uint32_t N, uint32_t M, double *gli, float *cpro);
int ApplyPropagator(double a, double b, double gam, double thickness, double E, double Xtilt,
                    double Ytilt, uint32_t N, uint32_t M, double *gli, float *cpro);

/* Real-space atoms (PG_RS.cpp, Pot_RS.cpp).  Per pixel A = sum res occ and
 * B = sum res occ ads over the atoms whose box (radius atrad) covers it.  PG_*
 * multiply gli by the phase grating exp(-K B) exp(-i K A), K the relativistic
 * interaction constant at E volts; Potential_* add (A, B) to gli.  res is a
 * tabulated radial curve of the atom's type interpolated at r/dds ("curve"), or
 * the Doyle-Turner potential of Z = type with a per-atom Debye-Waller factor dw
 * ("DT_DW") or none ("DT_TV").  "DW" forms take fractional coordinates, "TV"
 * forms Angstrom; "periodic" forms wrap each atom's box over the cell edges,
 * "cutpot" forms clip it. */
#define MSL_MUSLIB_CURVE_ARGS                                                              \
    uint32_t N, uint32_t M, uint32_t Na, double *xx, double *yy, double *ads, double *occ, \
        int32_t *type, double *scatentryes, uint32_t Npoints, double dds, double *gli, float *cpro
#define MSL_MUSLIB_DTDW_ARGS                                                               \
    uint32_t N, uint32_t M, uint32_t Na, double *xx, double *yy, double *dw, double *ads,  \
        double *occ, int32_t *type, double *gli, float *cpro
#define MSL_MUSLIB_DTTV_ARGS                                                               \
    uint32_t N, uint32_t M, uint32_t Na, double *xx, double *yy, double *ads, double *occ, \
        int32_t *type, double *gli, float *cpro
int PG_rs_curve_DW_cutpot(double a, double b, double gam, double E, double atrad, MSL_MUSLIB_CURVE_ARGS);   /* PG_RS.cpp:57-119 */
int PG_rs_curve_TV_cutpot(double a, double b, double gam, double E, double atrad, MSL_MUSLIB_CURVE_ARGS);   /* :121-186 */
int PG_rs_DT_DW_cutpot(double a, double b, double gam, double E, double atrad, MSL_MUSLIB_DTDW_ARGS);       /* :188-241 */
int PG_rs_DT_TV_cutpot(double a, double b, double gam, double E, double atrad, MSL_MUSLIB_DTTV_ARGS);       /* :243-300 */
int PG_rs_curve_DW_periodic(double a, double b, double gam, double E, double atrad, MSL_MUSLIB_CURVE_ARGS); /* :304-452 */
int PG_rs_DT_DW_periodic(double a, double b, double gam, double E, double atrad, MSL_MUSLIB_DTDW_ARGS);     /* :454-598 */
int PG_rs_curve_TV_periodic(double a, double b, double gam, double E, double atrad, MSL_MUSLIB_CURVE_ARGS); /* :602-751 */
int PG_rs_DT_TV_periodic(double a, double b, double gam, double E, double atrad, MSL_MUSLIB_DTTV_ARGS);     /* :754-897 */
int Potential_rs_curve_DW_cutpot(double a, double b, double gam, double atrad, MSL_MUSLIB_CURVE_ARGS);      /* Pot_RS.cpp:5-55 */
int Potential_rs_curve_TV_cutpot(double a, double b, double gam, double atrad, MSL_MUSLIB_CURVE_ARGS);      /* :57-109 */
int Potential_rs_DT_DW_cutpot(double a, double b, double gam, double atrad, MSL_MUSLIB_DTDW_ARGS);          /* :111-155 */
int Potential_rs_DT_TV_cutpot(double a, double b, double gam, double atrad, MSL_MUSLIB_DTTV_ARGS);          /* :157-207 */
int Potential_rs_curve_DW_periodic(double a, double b, double gam, double atrad, MSL_MUSLIB_CURVE_ARGS);    /* :209-348 */
int Potential_rs_DT_DW_periodic(double a, double b, double gam, double atrad, MSL_MUSLIB_DTDW_ARGS);        /* :350-486 */
int Potential_rs_curve_TV_periodic(double a, double b, double gam, double atrad, MSL_MUSLIB_CURVE_ARGS);    /* :488-627 */
int Potential_rs_DT_TV_periodic(double a, double b, double gam, double atrad, MSL_MUSLIB_DTTV_ARGS);        /* :629-763 */
/* PG_RS.cpp:5-55: the curve grating of one atom over every pixel, K given. */
int PG_rs_curve_DW_cutpot_oneatom(double a, double b, double gam, double K, double atrad, uint32_t N,
                                  uint32_t M, double xx, double yy, double ads, double occ,
                                  double *scatentry, uint32_t Npoints, double dds, double *gli);

/* Reciprocal-space potential (Pot_rec_DT_DW.cpp:3-134, Pot_rec_curve_DW.cpp:7-164):
 * adds to gli, rows SL..EL-1 of an M-row grid (EL - SL rows of N complex
 * doubles), the Fourier coefficients of the atoms' potential on the
 * reflections (+-i Nmult, +-j Mmult) with i Nmult < N/2 and j Mmult < M/2:
 * sum over atoms of res(|g|/2) occ (1 + i ads) exp(-2 pi i (h x + k y)), res the
 * Doyle-Turner factor f(s) exp(-DW s^2) / cell area, or the type's curve. */
int Potential_rec_DT_DW(double a, double b, double gam, uint32_t Nmult, uint32_t Mmult, uint32_t N,
                        uint32_t M, uint32_t Na, uint32_t SL, uint32_t EL, double *xx, double *yy,
                        double *DW, double *ads, double *occ, int32_t *type, double *gli, float *cpro);
int Potential_rec_curve_DW(double a, double b, double gam, uint32_t Nmult, uint32_t Mmult, uint32_t N,
                           uint32_t M, uint32_t Na, uint32_t SL, uint32_t EL, double *xx, double *yy,
                           double *ads, double *occ, int32_t *type, double *scatentryes,
                           uint32_t Npoints, double dds, double *gli, float *cpro);

/* Doyle-Turner scattering factors and radial curves (Curves.cpp:3-81), host
 * code: i is Z (1..92).  scat_ampl_rs_DT_DW: projected potential at radius s;
 * scat_ampl_rs2_*: at squared radius s; CreatePots_rec_DT_DW / _rs_DT_DW fill
 * sc[Ntypes][Npoints] at s = 0, dds, 2 dds, ... (reciprocal with cell factor
 * _Vol / real space). */
double scat_ampl_rs_DT_DW(int i, double s, double dw);
double scat_ampl_rs2_DT_DW(int i, double s, double dw);
double scat_ampl_rs2_DT_DW0(int i, double s);
void CreatePots_rec_DT_DW(uint32_t Ntypes, uint32_t Npoints, double dds, int32_t *types, double *DW,
                          double _Vol, double *sc);
void CreatePots_rs_DT_DW(uint32_t Ntypes, uint32_t Npoints, double dds, int32_t *types, double *DW,
                         double *sc);

/* ------------------------------------------------- no-allocation variant */

/* msl_multislice for callers that may not allocate device memory -- for
 * instance code living inside an application whose own pool allocator owns
 * the GPU's memory, or a latency-critical loop in which a cudaMalloc/cudaFree
 * would stall the whole device.  No counterpart exists in the reference: it is
 * an addition of this library.
 *
 * Same arithmetic, kernels and launch sequence as msl_multislice, but no
 * context and no allocation of any kind: trans and psi must be device buffers
 * of the current device, owned by the caller; dz and layer_seq are host
 * arrays.  The twiddle, band-limit and propagator tables go into one
 * file-scope device array of MSL_NOALLOC_SCRATCH_BYTES that every GPU loading
 * the library keeps until exit.  Limits: sides up to MSL_NOALLOC_MAX_SIDE and
 * at most MSL_NOALLOC_MAX_LAYERS layers (ntrans); larger requests return
 * MSL_E_ARG / MSL_E_UNSUPPORTED without touching the device.
 *
 * Work runs on `stream` (a cudaStream_t, NULL for the default stream) and the
 * call waits for that stream before returning.  The first call on each device
 * looks up the array's device address (cudaGetSymbolAddress) with that device
 * current.  All calls share
 * the array: calls that overlap on the GPU (several host threads, several
 * streams of one device) race on it.  Errors are reported by the return code
 * only (there is no context to hold a message); a pass kernel that gives up a
 * bounded wait or finds its shared-memory layout wrong raises an error word
 * kept in the same array (cleared by every call), and the call then returns
 * MSL_E_CUDA. */
#define MSL_NOALLOC_MAX_SIDE 2048
#define MSL_NOALLOC_MAX_LAYERS 64
#define MSL_NOALLOC_SCRATCH_BYTES 2150656
int msl_multislice_noalloc(const msl_grid *grid, const msl_optics *optics, const float *trans,
                           int ntrans, const double *dz, const int *layer_seq, int nslice,
                           float *psi, int batch, int plane_wave, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* MSL_H */
