/*
 * Test infrastructure (oracle only; never linked into the product).
 *
 * A ctypes-callable driver around E. J. Kirkland's own CPU multislice code as
 * shipped in the reference (ImageSimulation/multislice: cfpix.cpp, slicelib.cpp),
 * compiled unchanged from the reference tree by oracle/ref/Makefile and linked
 * against the vendored FFTW 2.1.5 (float) through fftw3f_on_fftw2.c.
 *
 * What is the reference's code here: the FFT wrapper cfpix (fft = FFTW_BACKWARD
 * i.e. exp(+i..) unscaled; ifft = exp(-i..) scaled by 1/(nx*ny)), propagate()
 * (slicelib.cpp:744-790), freqn() (:433-463), vzatom() with bessk0/bessi0
 * (:2666-2716, :168, :210), wavelength() (:2795-2806) and sigma() (:2387-2412).
 *
 * What this file adds (restated from the reference's drivers, which cannot run
 * here as programs): the slice loop of mulslice.cpp:359-522 and :706-739 with the
 * potential handed in as numbers rather than TIFF files; the real-space binned
 * potential sum of LMultiSlice ModelPotential.cu:27-99 / :125-230 evaluated with
 * Kirkland's vzatom; and the C# STEM probe (MSProject.cs:458-514), checkpoint
 * detection (MSReuseCalculator.cs:36-92) and annular detector sum
 * (MSProject.cs:792-842), expressed in Kirkland's sign convention (the C# code
 * uses the complex-conjugate convention; all intensities are identical).
 */
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "cfpix.hpp"
#include "slicelib.hpp"
#include "floatTIFF.hpp"

extern double **fparams;   // slicelib.cpp:138
extern int feTableRead;    // slicelib.cpp:137

extern "C" {

/* Replace Kirkland's built-in fe table with a caller-supplied one (the
 * reference's FPARAMS.DAT values, 12 numbers per Z in the order
 * a1 b1 a2 b2 a3 b3 c1 d1 c2 d2 c3 d3).  tab holds rows Z = 0..103. */
int kref_set_fparams(const double *tab, int nz)
{
    (void)vzatom(6, 1.0);  // forces ReadfeTable() to allocate fparams
    if (feTableRead != 1 || fparams == NULL) return -1;
    for (int Z = 1; Z < nz && Z <= 103; Z++)
        for (int i = 0; i < 12; i++) fparams[Z][i] = tab[Z * 12 + i];
    return 0;
}

double kref_vzatom(int Z, double r) { return vzatom(Z, r); }
double kref_wavelength(double kev) { return wavelength(kev); }
double kref_sigma(double kev) { return sigma(kev); }

/* Projected potential V_z (volt-Angstrom) per slice, layout [slice][ix][iy].
 * Binning: slice index = floor(z / dz), dz = cz_total / nslice; atoms outside
 * [0, cz_total) are dropped, as in ModelPotential.cu:63-71.  Minimum image on
 * |dx|, |dy| and the strict cutoff r < radius follow ModelPotential.cu:154-203.
 * Only pixels inside each atom's periodic bounding box are visited; all others
 * have r >= radius, so the sum equals the reference's all-pixel scan. */
int kref_potential(int natom, const double *x, const double *y, const double *z,
                   const int *Znum, double ax, double by, double cz_total,
                   int nx, int ny, int nslice, double radius, double *vout)
{
    if (2.0 * radius >= ax || 2.0 * radius >= by) return -1;
    const double dz = cz_total / nslice;
    const double dxp = ax / nx, dyp = by / ny;
    const double hax = ax / 2.0, hby = by / 2.0;
    std::memset(vout, 0, sizeof(double) * (size_t)nslice * nx * ny);
    for (int a = 0; a < natom; a++) {
        int kz = (int)std::floor(z[a] / dz);
        if (z[a] < 0.0 || kz < 0 || kz >= nslice) continue;
        double xa = x[a] - ax * std::floor(x[a] / ax);
        double ya = y[a] - by * std::floor(y[a] / by);
        int ix0 = (int)std::floor((xa - radius) / dxp) - 1;
        int ix1 = (int)std::ceil((xa + radius) / dxp) + 1;
        int iy0 = (int)std::floor((ya - radius) / dyp) - 1;
        int iy1 = (int)std::ceil((ya + radius) / dyp) + 1;
        if (ix1 - ix0 + 1 > nx) { ix0 = 0; ix1 = nx - 1; }
        if (iy1 - iy0 + 1 > ny) { iy0 = 0; iy1 = ny - 1; }
        double *vs = vout + (size_t)kz * nx * ny;
        for (int jx = ix0; jx <= ix1; jx++) {
            int ix = ((jx % nx) + nx) % nx;
            double ddx = std::fabs(xa - ix * dxp);
            if (ddx >= hax) ddx = ax - ddx;
            for (int jy = iy0; jy <= iy1; jy++) {
                int iy = ((jy % ny) + ny) % ny;
                double ddy = std::fabs(ya - iy * dyp);
                if (ddy >= hby) ddy = by - ddy;
                double r = std::sqrt(ddx * ddx + ddy * ddy);
                if (r < radius) {
                    if (r < 1.0e-10) r = 1.0e-10;
                    vs[(size_t)ix * ny + iy] += vzatom(Znum[a], r);
                }
            }
        }
    }
    return 0;
}

/* Shared set-up of mulslice.cpp:359-522: transmission functions (band-limited
 * by fft -> mask -> ifft) and the separable propagator tables per layer. */
struct KSetup {
    int nx, ny, nlayer;
    float wavlen, mm0, k2max;
    std::vector<float> kx, kx2, xpos, ky, ky2, ypos;
    std::vector<std::vector<float>> pxr, pxi, pyr, pyi;
    cfpix *trans;
};

static void ksetup(KSetup &S, int nx, int ny, double ax_d, double by_d, double v0_d,
                   int nlayer, const double *vz, const double *cz_d, double ctiltx_d,
                   double ctilty_d)
{
    S.nx = nx; S.ny = ny; S.nlayer = nlayer;
    float v0 = (float)v0_d, ax = (float)ax_d, by = (float)by_d;
    float pi = (float)(4.0 * atan(1.0));
    S.mm0 = 1.0F + v0 / 511.0F;
    S.wavlen = (float)wavelength(v0);
    const double sig = sigma(v0) / 1000.0;  // rad / (V A)
    S.trans = new cfpix[nlayer];
    float scale = S.wavlen * S.mm0;
    for (int l = 0; l < nlayer; l++) {
        S.trans[l].resize(nx, ny);
        if (l == 0) S.trans[l].init(0, 1);
        else S.trans[l].copyInit(S.trans[0]);
        const double *v = vz + (size_t)l * nx * ny;
        for (int ix = 0; ix < nx; ix++)
            for (int iy = 0; iy < ny; iy++) {
                // the potential "file" value whose lambda*mm0 multiple is sigma*V_z
                float vfile = (float)(sig * v[(size_t)ix * ny + iy] / ((double)S.wavlen * S.mm0));
                float ph = scale * vfile;
                S.trans[l].re(ix, iy) = (float)cos(ph);
                S.trans[l].im(ix, iy) = (float)sin(ph);
            }
    }
    S.kx.resize(nx); S.kx2.resize(nx); S.xpos.resize(nx);
    S.ky.resize(ny); S.ky2.resize(ny); S.ypos.resize(ny);
    freqn(S.kx.data(), S.kx2.data(), S.xpos.data(), nx, ax);
    freqn(S.ky.data(), S.ky2.data(), S.ypos.data(), ny, by);

    const float BW = 2.0F / 3.0F;
    float k2max = nx / (2.0F * ax);
    float tctx = ny / (2.0F * by);
    if (tctx < k2max) k2max = tctx;
    k2max = BW * k2max;
    k2max = k2max * k2max;
    S.k2max = k2max;
    tctx = (float)(2.0 * tan(ctiltx_d));
    float tcty = (float)(2.0 * tan(ctilty_d));

    S.pxr.assign(nlayer, std::vector<float>(nx));
    S.pxi.assign(nlayer, std::vector<float>(nx));
    S.pyr.assign(nlayer, std::vector<float>(ny));
    S.pyi.assign(nlayer, std::vector<float>(ny));
    for (int l = 0; l < nlayer; l++) {
        float czl = (float)cz_d[l];
        float sc = pi * czl;
        double t;
        for (int ix = 0; ix < nx; ix++) {
            t = sc * (S.kx2[ix] * S.wavlen - S.kx[ix] * tctx);
            S.pxr[l][ix] = (float)cos(t);
            S.pxi[l][ix] = (float)-sin(t);
        }
        for (int iy = 0; iy < ny; iy++) {
            t = sc * (S.ky2[iy] * S.wavlen - S.ky[iy] * tcty);
            S.pyr[l][iy] = (float)cos(t);
            S.pyi[l][iy] = (float)-sin(t);
        }
        S.trans[l].fft();
        for (int ix = 0; ix < nx; ix++)
            for (int iy = 0; iy < ny; iy++) {
                float k2 = S.ky2[iy] + S.kx2[ix];
                if (!(k2 < k2max)) S.trans[l].re(ix, iy) = S.trans[l].im(ix, iy) = 0.0F;
            }
        S.trans[l].ifft();
    }
}

static void kfree(KSetup &S) { delete[] S.trans; }

/* Band-limited transmission functions only: out [nlayer][nx][ny][2] float. */
int kref_transmission(int nx, int ny, double ax, double by, double v0, int nlayer,
                      const double *vz, const double *cz, float *out)
{
    KSetup S;
    ksetup(S, nx, ny, ax, by, v0, nlayer, vz, cz, 0.0, 0.0);
    for (int l = 0; l < nlayer; l++)
        for (int ix = 0; ix < nx; ix++)
            for (int iy = 0; iy < ny; iy++) {
                size_t o = (((size_t)l * nx + ix) * ny + iy) * 2;
                out[o] = S.trans[l].re(ix, iy);
                out[o + 1] = S.trans[l].im(ix, iy);
            }
    kfree(S);
    return 0;
}

/* Coherent CTEM multislice of mulslice.cpp:706-739.  wave_in may be NULL for
 * an untilted plane wave of amplitude 1.  wave_out [nx][ny][2]; intensity
 * [nslice] receives the per-slice integrated intensity (mulslice.cpp:727-733). */
int kref_ctem(int nx, int ny, double ax, double by, double v0, int nlayer,
              const double *vz, const double *cz, int nslice, const int *layer_seq,
              double ctiltx, double ctilty, const float *wave_in, float *wave_out,
              double *intensity)
{
    KSetup S;
    ksetup(S, nx, ny, ax, by, v0, nlayer, vz, cz, ctiltx, ctilty);
    cfpix wave;
    wave.resize(nx, ny);
    wave.copyInit(S.trans[0]);
    for (int ix = 0; ix < nx; ix++)
        for (int iy = 0; iy < ny; iy++) {
            if (wave_in) {
                wave.re(ix, iy) = wave_in[((size_t)ix * ny + iy) * 2];
                wave.im(ix, iy) = wave_in[((size_t)ix * ny + iy) * 2 + 1];
            } else {
                wave.re(ix, iy) = 1.0F;
                wave.im(ix, iy) = 0.0F;
            }
        }
    float scale = 1.0F / (((float)nx) * ((float)ny));
    for (int islice = 0; islice < nslice; islice++) {
        int l = layer_seq[islice];
        wave *= S.trans[l];
        wave.fft();
        propagate(wave, S.pxr[l].data(), S.pxi[l].data(), S.pyr[l].data(), S.pyi[l].data(),
                  S.kx2.data(), S.ky2.data(), S.k2max, nx, ny);
        wave.ifft();
        double sum = 0.0;
        for (int ix = 0; ix < nx; ix++)
            for (int iy = 0; iy < ny; iy++)
                sum += wave.re(ix, iy) * wave.re(ix, iy) + wave.im(ix, iy) * wave.im(ix, iy);
        if (intensity) intensity[islice] = sum * scale;
    }
    for (int ix = 0; ix < nx; ix++)
        for (int iy = 0; iy < ny; iy++) {
            wave_out[((size_t)ix * ny + iy) * 2] = wave.re(ix, iy);
            wave_out[((size_t)ix * ny + iy) * 2 + 1] = wave.im(ix, iy);
        }
    kfree(S);
    return 0;
}

/* STEM scan: for each probe position build the converged probe in reciprocal
 * space (MSProject.cs:458-514), inverse transform, run the slice loop and, after
 * the propagator of every checkpoint slice (MSReuseCalculator.cs:67-78), sum
 * |Psi(k)|^2 over each annulus kin^2 <= s <= kout^2 (MSProject.cs:792-842).
 *
 * probe_xy [nprobe][2] in Angstrom; det_k [ndet][2] = (k_inner, k_outer) in 1/A;
 * checkpoints: ascending slice indices (0-based) after which detection happens.
 * det_out [nprobe][ncheck][ndet]. */
int kref_stem(int nx, int ny, double ax, double by, double v0, int nlayer,
              const double *vz, const double *cz, int nslice, const int *layer_seq,
              double kap_in, double kap_out, double df, double cs, int nprobe,
              const double *probe_xy, int ndet, const double *det_k, int ncheck,
              const int *checkpoints, double *det_out)
{
    KSetup S;
    ksetup(S, nx, ny, ax, by, v0, nlayer, vz, cz, 0.0, 0.0);
    const double lam = wavelength(v0);
    const double pi = 4.0 * atan(1.0);
    const double smin = kap_in * kap_in, smax = kap_out * kap_out;
    cfpix wave;
    wave.resize(nx, ny);
    wave.copyInit(S.trans[0]);
    for (int p = 0; p < nprobe; p++) {
        const double fx = probe_xy[2 * p] / ax, fy = probe_xy[2 * p + 1] / by;
        for (int ix = 0; ix < nx; ix++) {
            int i = ix < nx / 2 ? ix : ix - nx;
            double kxv = (double)i / ax;
            for (int iy = 0; iy < ny; iy++) {
                int j = iy < ny / 2 ? iy : iy - ny;
                double kyv = (double)j / by;
                double s = kxv * kxv + kyv * kyv;
                if (s >= smin && s <= smax) {
                    double chi = pi * (lam * df * s + 0.5 * cs * lam * lam * lam * s * s);
                    double ph = 2.0 * pi * ((double)i * fx + (double)j * fy) - chi;
                    wave.re(ix, iy) = (float)cos(ph);
                    wave.im(ix, iy) = (float)sin(ph);
                } else {
                    wave.re(ix, iy) = 0.0F;
                    wave.im(ix, iy) = 0.0F;
                }
            }
        }
        wave.ifft();
        int ic = 0;
        for (int islice = 0; islice < nslice && ic < ncheck; islice++) {
            int l = layer_seq[islice];
            wave *= S.trans[l];
            wave.fft();
            propagate(wave, S.pxr[l].data(), S.pxi[l].data(), S.pyr[l].data(), S.pyi[l].data(),
                      S.kx2.data(), S.ky2.data(), S.k2max, nx, ny);
            if (checkpoints[ic] == islice) {
                for (int d = 0; d < ndet; d++) {
                    double dmin = det_k[2 * d] * det_k[2 * d];
                    double dmax = det_k[2 * d + 1] * det_k[2 * d + 1];
                    double acc = 0.0;
                    for (int ix = 0; ix < nx; ix++) {
                        int i = ix < nx / 2 ? ix : ix - nx;
                        double kxv = (double)i / ax;
                        for (int iy = 0; iy < ny; iy++) {
                            int j = iy < ny / 2 ? iy : iy - ny;
                            double kyv = (double)j / by;
                            double s = kxv * kxv + kyv * kyv;
                            if (s <= dmax && s >= dmin) {
                                double wr = wave.re(ix, iy), wi = wave.im(ix, iy);
                                acc += wr * wr + wi * wi;
                            }
                        }
                    }
                    det_out[((size_t)p * ncheck + ic) * ndet + d] = acc;
                }
                ic++;
            }
            if (ic < ncheck) wave.ifft();
        }
    }
    kfree(S);
    return 0;
}

/* The reference's aberration function chi() (slicelib.cpp:258-323) as compiled
 * from slicelib.cpp: p holds the aberration coefficients at the slicelib
 * parameter indices (pCS, pDEFOCUS, pC12a, ...; Angstrom; kref_nparam() floats),
 * (alx, aly) the angles in radians; returns w, chi = 2 pi w / lambda. */
static const int kChiParams = 64;  // chi() reads indices up to pC56b = 56
double kref_chi(const float *p, double alx, double aly, int multiMode)
{
    std::vector<float> q(p, p + kChiParams);
    return chi(q.data(), alx, aly, multiMode);
}
int kref_nparam(void) { return kChiParams; }
int kref_param_index(int which)
{
    switch (which) {
        case 0: return pCS;
        case 1: return pDEFOCUS;
        case 2: return pC12a;
        case 3: return pC12b;
        case 4: return pC23a;
        case 5: return pC23b;
        default: return -1;
    }
}

/* Partial-coherence CTEM image of mulslice.cpp:539-676 (its lpartl == 1 branch),
 * restated with the same variable types (float images and angles, double chi,
 * float defocus weights) and driven by the reference's cfpix fft / ifft and
 * propagate: every illumination angle (qx, qy) = (iqx rx, iqy ry) with
 * q2min <= q2 <= q2max starts a tilted plane wave (mulslice.cpp:583-590), runs the
 * slice loop, and its spectrum is imaged through exp(-i chi) inside the
 * objective aperture for defocus df0 + idf dfdelt, |idf| <= 2.5 sigmaf / dfdelt,
 * weighted exp(-(idf dfdelt / sigmaf)^2 / 2); pix [nx][ny] is normalised by
 * nillum * sum of weights.  cs_mm in mm, df0 / sigmaf / dfdelt / dfa2 / dfa3 in
 * Angstrom, angles acmin / acmax / aobj in mrad as mulslice reads them
 * (mulslice.cpp:233-283), dfa2phi / dfa3phi in degrees.  *nillum_out receives
 * the angle count. */
int kref_partial_coherence(int nx, int ny, double ax_d, double by_d, double v0_d, int nlayer,
                           const double *vz, const double *cz, int nslice, const int *layer_seq,
                           double cs_mm, double df0_d, double sigmaf_d, double dfdelt_d, double aobj_mrad,
                           double acmin_mrad, double acmax_mrad, double dfa2_d, double dfa2phi_deg,
                           double dfa3_d, double dfa3phi_deg, float *pix_out, int *nillum_out)
{
    KSetup S;
    ksetup(S, nx, ny, ax_d, by_d, v0_d, nlayer, vz, cz, 0.0, 0.0);
    const float pi = (float)(4.0 * atan(1.0));
    const float ax = (float)ax_d, by = (float)by_d;
    const float wavlen = S.wavlen;
    // mulslice.cpp reads these as floats and converts the units (:233-283)
    float Cs = (float)cs_mm * 1.0e7F;
    float df0 = (float)df0_d, sigmaf = (float)sigmaf_d, dfdelt = (float)dfdelt_d;
    float aobj = (float)aobj_mrad * 0.001F, acmin = (float)acmin_mrad * 0.001F,
          acmax = (float)acmax_mrad * 0.001F;
    float dfa2 = (float)dfa2_d, dfa3 = (float)dfa3_d;
    float dfa2phi = (float)dfa2phi_deg * pi / 180.0F, dfa3phi = (float)dfa3phi_deg * pi / 180.0F;
    float rx = 1.0F / ax, ry = 1.0F / by;
    if (sigmaf <= 0.0F) { sigmaf = 0.0F; dfdelt = 1.0F; }   // one defocus value

    cfpix wave, ctemp;
    wave.resize(nx, ny);
    wave.copyInit(S.trans[0]);
    ctemp.resize(nx, ny);
    ctemp.copyInit(S.trans[0]);
    std::vector<float> pix((size_t)nx * ny, 0.0F);

    float scale = 1.0F / (((float)nx) * ((float)ny));
    int ndf = (int)((2.5F * sigmaf) / dfdelt);
    int nacx = (int)((acmax / (wavlen * rx)) + 1.5F);
    int nacy = (int)((acmax / (wavlen * ry)) + 1.5F);
    float q2max = acmax / wavlen;
    q2max = q2max * q2max;
    float q2min = acmin / wavlen;
    q2min = q2min * q2min;
    float k2maxo = aobj / wavlen;
    k2maxo = k2maxo * k2maxo;
    double chi1 = pi * wavlen;
    double chi2 = 0.5 * Cs * wavlen * wavlen;
    long nillum = 0;
    float sumdf = 0.0F;
    for (int iqy = -nacy; iqy <= nacy; iqy++) {
        float qy = iqy * ry;
        float qy2 = qy * qy;
        for (int iqx = -nacx; iqx <= nacx; iqx++) {
            float qx = iqx * rx;
            float q2 = qx * qx + qy2;
            if ((q2 <= q2max) && (q2 >= q2min)) {
                nillum += 1;
                for (int ix = 0; ix < nx; ix++)
                    for (int iy = 0; iy < ny; iy++) {
                        double t = 2.0 * pi * (qx * S.xpos[ix] + qy * S.ypos[iy]);
                        wave.re(ix, iy) = (float)cos(t);
                        wave.im(ix, iy) = (float)sin(t);
                    }
                for (int islice = 0; islice < nslice; islice++) {
                    int l = layer_seq[islice];
                    wave *= S.trans[l];
                    wave.fft();
                    propagate(wave, S.pxr[l].data(), S.pxi[l].data(), S.pyr[l].data(), S.pyi[l].data(),
                              S.kx2.data(), S.ky2.data(), S.k2max, nx, ny);
                    wave.ifft();
                }
                wave.fft();
                sumdf = 0.0F;
                for (int idf = -ndf; idf <= ndf; idf++) {
                    float df = df0 + idf * dfdelt;
                    for (int ix = 0; ix < nx; ix++)
                        for (int iy = 0; iy < ny; iy++) {
                            float k2 = S.kx2[ix] + S.ky2[iy];
                            if (k2 <= k2maxo) {
                                double phi = atan2(S.ky[iy], S.kx[ix]);
                                double chi = chi1 * k2 * (chi2 * k2 - df + dfa2 * sin(2.0 * (phi - dfa2phi)) +
                                                          2.0F * dfa3 * wavlen * sqrt(k2) *
                                                              sin(3.0 * (phi - dfa3phi)) / 3.0);
                                float tr = (float)cos(chi);
                                float ti = (float)-sin(chi);
                                float wr = wave.re(ix, iy);
                                float wi = wave.im(ix, iy);
                                ctemp.re(ix, iy) = wr * tr - wi * ti;
                                ctemp.im(ix, iy) = wr * ti + wi * tr;
                            } else {
                                ctemp.re(ix, iy) = 0.0F;
                                ctemp.im(ix, iy) = 0.0F;
                            }
                        }
                    ctemp.ifft();
                    float pdf = 1.0F;
                    if (sigmaf > 0.0F) {
                        double xdf = (double)((df - df0) / sigmaf);
                        pdf = (float)exp(-0.5F * xdf * xdf);
                    }
                    sumdf += pdf;
                    for (int ix = 0; ix < nx; ix++)
                        for (int iy = 0; iy < ny; iy++) {
                            float x = ctemp.re(ix, iy), y = ctemp.im(ix, iy);
                            pix[(size_t)ix * ny + iy] += pdf * (x * x + y * y);
                        }
                }
            }
        }
    }
    scale = 1.0F / (((float)nillum) * sumdf);
    for (size_t i = 0; i < pix.size(); i++) pix_out[i] = pix[i] * scale;
    if (nillum_out) *nillum_out = (int)nillum;
    kfree(S);
    return 0;
}

// floatTIFF round trip: the reference's own reader and writer of Kirkland's
// TIFF files (floatTIFF.cpp:324-350, :1263-1840).  data is [ny][nx] (row iy,
// column ix); params holds PMAX = 512 floats.
int kref_tiff_write(const char *path, const float *data, int nx, int ny, int npix, const float *params,
                    float rmin, float rmax, float imin, float imax, float dx, float dy) {
    floatTIFF f;
    f.resize(nx, ny);
    f.setnpix(npix);
    for (int i = 0; i < f.maxParam(); ++i) f.setParam(i, params[i]);
    for (int iy = 0; iy < ny; ++iy)
        for (int ix = 0; ix < nx; ++ix) f(ix, iy) = data[(size_t)iy * nx + ix];
    return f.write(path, rmin, rmax, imin, imax, dx, dy);
}

int kref_tiff_read(const char *path, float *data, int cap, int *nx, int *ny, int *npix, float *params) {
    floatTIFF f;
    const int rc = f.read(path);
    if (rc != 1) return rc;
    *nx = f.nx();
    *ny = f.ny();
    *npix = f.getnpix();
    for (int i = 0; i < f.maxParam(); ++i) params[i] = f.getParam(i);
    if ((long)(*nx) * (*ny) > cap) return -100;
    for (int iy = 0; iy < *ny; ++iy)
        for (int ix = 0; ix < *nx; ++ix) data[(size_t)iy * (*nx) + ix] = f(ix, iy);
    return 1;
}

// The reference's stacking-sequence parser (slicelib.cpp:620-720).
int kref_parlay(const char *c, int *islice, int nsmax, int lmax, int *nslice) {
    return parlay(c, islice, nsmax, lmax, nslice, 0);
}

}  // extern "C"
