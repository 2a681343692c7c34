// Muslib-shaped exports: the C entry points the reference's C# STEM driver binds
// through P/Invoke (MSProjectReuse.cs:24-93, MSUseOnceCalculator.cs:15-78), with
// identical argument lists, so that driver runs unchanged against this library.
// Windows ULONG / LONG are 32-bit, hence uint32_t / int32_t here.  Buffers are
// the caller's host arrays in the C# layout: N x M complex doubles, row j (y)
// major, (re, im) interleaved: element (i, j) at gli[2 * (j * N + i)].
//
// Each call runs on the current CUDA device: it copies gli in, computes with
// FP64 kernels, copies it back, and writes *cpro = 100 (the reference's progress
// output).  Return value 0 on success (the reference defines no other codes);
// here a CUDA failure or an invalid size returns -1.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include <algorithm>
#include <mutex>
#include <vector>

namespace {

// The C# driver's wavelength and interaction-constant forms (E in volts):
// Propagator.cpp:17, PG_RS.cpp:317-318.
__host__ __device__ inline double cs_lambda(double E) {
    return 0.387818 / sqrt(E / 1000.0 * (1.0 + 0.978459e-3 * E / 1000));
}

__global__ void propagator_kernel(double A, double B, double cos_g, double GK, double XTG, double YTG,
                                  double smax, uint32_t N, uint32_t M, double *gli, int apply) {
    const uint32_t ii = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t jj = blockIdx.y;
    if (ii >= N || jj >= M) return;
    const long j = jj < M / 2 ? (long)jj : (long)jj - (long)M;
    const long i = ii < N / 2 ? (long)ii : (long)ii - (long)N;
    const double y = (double)j * B, y2 = y * y, ycos = -2.0 * y * cos_g;
    const double x = (double)i * A;
    const double s = x * (x + ycos) + y2;
    double *p = gli + 2 * ((size_t)jj * N + ii);
    if (s >= smax) {
        p[0] = 0.0;
        p[1] = 0.0;
        return;
    }
    const double con = GK * s - XTG * x - YTG * y;
    double sn, cn;
    sincos(con, &sn, &cn);
    if (apply) {
        const double wr = p[0], wi = p[1];
        p[0] = wr * cn - wi * sn;
        p[1] = wr * sn + wi * cn;
    } else {
        p[0] = cn;
        p[1] = sn;
    }
}

int propagator(double a, double b, double gam, double thickness, double E, double Xtilt, double Ytilt,
               uint32_t N, uint32_t M, double *gli, float *cpro, int apply) {
    if (cpro) *cpro = 0;
    if (!gli || N == 0 || M == 0 || !(a > 0) || !(b > 0)) return -1;
    const double A = 1.0 / (a * sin(gam)), B = 1.0 / (b * sin(gam));
    const double lambda = cs_lambda(E);
    const double GK = M_PI * lambda * thickness;
    double smax = fmin((double)N * 0.5 / a, (double)M * 0.5 / b);
    smax *= smax;
    const double XTG = 2.0 * M_PI * thickness * tan(Xtilt), YTG = 2.0 * M_PI * thickness * tan(Ytilt);
    const size_t bytes = sizeof(double) * 2 * (size_t)N * M;
    double *d = nullptr;
    if (cudaMalloc(&d, bytes) != cudaSuccess) return -1;
    int rc = 0;
    if (apply && cudaMemcpy(d, gli, bytes, cudaMemcpyHostToDevice) != cudaSuccess) rc = -1;
    if (!rc) {
        dim3 grid((N + 255) / 256, M);
        propagator_kernel<<<grid, 256>>>(A, B, cos(gam), GK, XTG, YTG, smax, N, M, d, apply);
        if (cudaGetLastError() != cudaSuccess ||
            cudaMemcpy(gli, d, bytes, cudaMemcpyDeviceToHost) != cudaSuccess)
            rc = -1;
    }
    cudaFree(d);
    if (!rc && cpro) *cpro = 100;
    return rc;
}

// Doyle & Turner (1968) four-Gaussian scattering factors, row Z = a1 b1 .. a4 b4
// (the Muslib bank of Curves.cpp:86-179).
constexpr int kDTRows = 93;
const double h_dt[kDTRows][8] = {
#include "msl_doyle_turner.inc"
};
__constant__ double c_dt[kDTRows][8];

// Curves.cpp:3-10: f(s) = sum_j a_j exp(-b_j s^2).
__host__ __device__ inline double dt_rec(const double (*tab)[8], int z, double s) {
    double sf = 0;
    s *= s;
    for (int j = 0; j < 4; ++j) sf += tab[z][2 * j] * exp(-tab[z][2 * j + 1] * s);
    return sf;
}

// Curves.cpp:23-32: projected potential at squared radius r2, Debye-Waller
// broadened: 4 pi sum_j a_j / (b_j + dw) exp(-4 pi^2 r2 / (b_j + dw)), b_j > 0.
__host__ __device__ inline double dt_rs2(const double (*tab)[8], int z, double r2, double dw) {
    double sf = 0;
    r2 *= -4.0 * M_PI * M_PI;
    for (int j = 0; j < 4; ++j) {
        const double bj = tab[z][2 * j + 1];
        if (bj > 0) sf += tab[z][2 * j] / (bj + dw) * exp(r2 / (bj + dw));
    }
    return sf * 4 * M_PI;
}

// Once per device (constant memory is per device), under a lock.
bool dt_upload() {
    static std::mutex mu;
    static bool done[64] = {};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return false;
    std::lock_guard<std::mutex> lock(mu);
    if (done[dev]) return true;
    if (cudaMemcpyToSymbol(c_dt, h_dt, sizeof(h_dt)) != cudaSuccess) return false;
    done[dev] = true;
    return true;
}

// ------------------------------------------------------------------ real space
// The sixteen real-space exports of PG_RS.cpp / Pot_RS.cpp differ in three
// choices, kept as flags here:
//  * radial source: a tabulated curve per type (linear interpolation at r/dds,
//    nothing beyond the curve) or the Doyle-Turner sum at r^2 for Z = type with
//    a per-atom Debye-Waller term ("DT_DW") or none ("DT_TV");
//  * coordinates: fractional ("DW" names) or Angstrom ("TV" names), each with
//    its own integer box bounds, reproduced formula by formula below;
//  * periodic (nine image rectangles, PG_RS.cpp:333-420) or clipped at the
//    cell edge ("cutpot").
// Per pixel the kernel accumulates A = sum res occ and B = sum res occ ads in
// FP64; the phase grating then multiplies gli by exp(-K B)(cos K A - i sin K A)
// (PG_RS.cpp:433-441, the product over atoms of the per-atom factors), the
// potential adds (A, B) to gli (Pot_RS.cpp:44-46).
struct Rect {
    int32_t ib, ie, jb, je;
    double x0, y0;
};

enum RsSource : int { RS_CURVE = 0, RS_DT_DW = 1, RS_DT_TV = 2 };

struct RsCall {
    double a, b, gam, K, atrad;
    uint32_t N, M, Na;
    const double *xx, *yy, *dw, *ads, *occ;
    const int32_t *type;
    const double *curves;
    uint32_t Npoints;
    double dds;
    double *gli;
    float *cpro;
    int source;        // RsSource
    bool angstrom;     // "TV" coordinates
    bool periodic;
    bool phase_grating;
    bool whole_grid;   // one atom over every pixel, PG_RS.cpp:26-30
};

__global__ void rs_accumulate_kernel(const Rect *rects, const int32_t *atom_of, const double *occ,
                                     const double *ads, const double *dw, const int32_t *type,
                                     const double *curves, uint32_t Npoints, double dds, int source,
                                     double dxa, double dyb, double cos_g, uint32_t N, double *A, double *Bacc) {
    const Rect r = rects[blockIdx.x];
    const int k = atom_of[blockIdx.x];
    const int tk = type[k];
    const double o = occ[k], ad = ads[k];
    const double dwk = source == RS_DT_DW ? dw[k] : 0.0;
    const double *curk = curves ? curves + (size_t)tk * Npoints : nullptr;
    const int w = r.ie - r.ib, h = r.je - r.jb;
    if (w <= 0 || h <= 0) return;
    for (int idx = threadIdx.x; idx < w * h; idx += blockDim.x) {
        const int j = r.jb + idx / w, i = r.ib + idx % w;
        const double y = __dsub_rn(__dmul_rn(j, dyb), r.y0), x = __dsub_rn(__dmul_rn(i, dxa), r.x0);
        // x (x + 2 y cos) + y^2, rounded step by step as the reference's C
        const double r2 = __dadd_rn(__dmul_rn(x, __dadd_rn(x, __dmul_rn(2 * y, cos_g))), __dmul_rn(y, y));
        double res;
        if (source == RS_CURVE) {
            const double ar2 = sqrt(r2) / dds;
            const double fl = floor(ar2);
            if (fl >= (double)(Npoints - 1)) continue;
            const uint32_t jjj = (uint32_t)fl;
            res = curk[jjj] + (curk[jjj + 1] - curk[jjj]) * (ar2 - jjj);
        } else {
            res = dt_rs2(c_dt, tk, r2, dwk);
        }
        const size_t p = (size_t)j * N + i;
        atomicAdd(A + p, res * o);
        atomicAdd(Bacc + p, res * o * ad);
    }
}

// Phase grating (PG_RS.cpp:434-441): gli *= exp(-K B) (cos K A - i sin K A).
__global__ void pg_apply_kernel(const double *A, const double *Bacc, double K, size_t n, double *gli) {
    const size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    double sn, cn;
    sincos(K * A[p], &sn, &cn);
    const double aI = exp(-K * Bacc[p]);
    const double rr = cn * aI, ri = -sn * aI;
    const double wr = gli[2 * p], wi = gli[2 * p + 1];
    gli[2 * p] = wr * rr - wi * ri;
    gli[2 * p + 1] = wr * ri + wi * rr;
}

// Potential (Pot_RS.cpp:44-45): gli += (A, B).
__global__ void pot_apply_kernel(const double *A, const double *Bacc, size_t n, double *gli) {
    const size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    gli[2 * p] += A[p];
    gli[2 * p + 1] += Bacc[p];
}

// Windows min(long, ULONG) compares unsigned: a negative bound becomes n.
inline long umin(long v, long n) { return (v >= 0 && v < n) ? v : n; }
inline long smax0(long v) { return v > 0 ? v : 0; }
inline long trunc_nonneg(double v) { return v > 0 ? (long)v : 0; }

// The pixel rectangles of atom k, formula by formula as the variant writes them.
void rs_rects(const RsCall &c, uint32_t k, double drax, double dray, std::vector<Rect> &out) {
    const long N = (long)c.N, M = (long)c.M;
    const double xk = c.xx[k], yk = c.yy[k], a = c.a, b = c.b;
    const double X = c.angstrom ? xk : xk * a, Y = c.angstrom ? yk : yk * b;
    auto add = [&](long ib, long ie, long jb, long je, double x0, double y0) {
        out.push_back({(int32_t)ib, (int32_t)ie, (int32_t)jb, (int32_t)je, x0, y0});
    };
    if (c.whole_grid) {
        add(0, N, 0, M, X, Y);
        return;
    }
    if (!c.periodic) {
        long ib, ie, jb, je;
        if (!c.angstrom) {             // PG_RS.cpp:81-84
            ib = smax0((long)((xk - drax) * c.N));
            ie = umin((long)((xk + drax) * c.N), N);
            jb = smax0((long)((yk - dray) * c.M));
            je = umin((long)((yk + dray) * c.M), M);
        } else if (c.source == RS_CURVE) {   // PG_RS.cpp:149-152: (long)(q) / a, then truncated
            ib = trunc_nonneg((double)(long)((xk - drax) * c.N) / a);
            ie = trunc_nonneg(fmin((double)(long)((xk + drax) * c.N) / a, (double)c.N));
            jb = trunc_nonneg((double)(long)((yk - dray) * c.M) / b);
            je = trunc_nonneg(fmin((double)(long)((yk + dray) * c.M) / b, (double)c.M));
        } else {                       // PG_RS.cpp:269-272: (long)(q / a)
            ib = smax0((long)((xk - drax) * c.N / a));
            ie = umin((long)((xk + drax) * c.N / a), N);
            jb = smax0((long)((yk - dray) * c.M / b));
            je = umin((long)((yk + dray) * c.M / b), M);
        }
        add(ib, ie, jb, je, X, Y);
        return;
    }
    long ibb, iee, jbb, jee;
    if (!c.angstrom) {                 // PG_RS.cpp:327-330
        ibb = (long)((xk - drax) * c.N);
        iee = (long)((xk + drax) * c.N);
        jbb = (long)((yk - dray) * c.M);
        jee = (long)((yk + dray) * c.M);
    } else {                           // PG_RS.cpp:625-628
        ibb = (long)((xk - drax) / a * c.N);
        iee = (long)((xk + drax) / a * c.N);
        jbb = (long)((yk - dray) / b * c.M);
        jee = (long)((yk + dray) / b * c.M);
    }
    const long ib0 = smax0(ibb), ie0 = umin(iee, N), jb0 = smax0(jbb), je0 = umin(jee, M);
    add(ib0, ie0, jb0, je0, X, Y);
    if (jbb < 0) add(ib0, ie0, jbb + M, M, X, Y + b);
    if (jee >= M) add(ib0, ie0, 0, jee - M + 1, X, Y - b);
    if (ibb < 0) add(ibb + N, N, jb0, je0, X + a, Y);
    if (iee >= N) add(0, iee - N + 1, jb0, je0, X - a, Y);
    if (ibb < 0 && jbb < 0) add(ibb + N, N, jbb + M, M, X + a, Y + b);
    if (iee >= N && jee >= M) add(0, iee - N + 1, 0, jee - M + 1, X - a, Y - b);
    if (iee >= N && jbb < 0) add(0, iee - N + 1, jbb + M, M, X - a, Y + b);
    if (ibb < 0 && jee >= M) add(ibb + N, N, 0, jee - M + 1, X + a, Y - b);
}

int rs_atoms(const RsCall &c) {
    if (!c.gli || c.N == 0 || c.M == 0 || !(c.a > 0) || !(c.b > 0)) return -1;
    const bool curve = c.source == RS_CURVE;
    if (curve && (c.Npoints < 2 || !(c.dds > 0))) return -1;
    if (c.Na > 0 && (!c.xx || !c.yy || !c.ads || !c.occ || !c.type || (curve && !c.curves) ||
                     (c.source == RS_DT_DW && !c.dw)))
        return -1;
    if (!curve && !dt_upload()) return -1;
    const double sin_gam = sin(c.gam), cos_gam = cos(c.gam);
    const double drax = c.angstrom ? c.atrad * sin_gam : c.atrad * sin_gam / c.a;
    const double dray = c.angstrom ? c.atrad * sin_gam : c.atrad * sin_gam / c.b;
    const double dxa = c.a / (double)c.N, dyb = c.b / (double)c.M;
    int32_t maxtype = 0;
    std::vector<Rect> rects;
    std::vector<int32_t> owner;
    for (uint32_t k = 0; k < c.Na; ++k) {
        if (c.type[k] < 0 || (!curve && c.type[k] >= kDTRows)) return -1;
        maxtype = c.type[k] > maxtype ? c.type[k] : maxtype;
        const size_t before = rects.size();
        rs_rects(c, k, drax, dray, rects);
        for (size_t q = before; q < rects.size(); ++q) {
            Rect &r = rects[q];
            // boxes wider than the cell would index outside it in the reference
            // (undefined there); here they are clipped to the grid
            if (r.ib < 0) r.ib = 0;
            if (r.jb < 0) r.jb = 0;
            if (r.ie > (int32_t)c.N) r.ie = (int32_t)c.N;
            if (r.je > (int32_t)c.M) r.je = (int32_t)c.M;
            owner.push_back((int32_t)k);
        }
    }
    const size_t n = (size_t)c.N * c.M;
    const size_t nc = curve ? (size_t)(maxtype + 1) * c.Npoints : 1;
    double *d_gli = nullptr, *d_ph = nullptr, *d_occ = nullptr, *d_ads = nullptr, *d_dw = nullptr,
           *d_cur = nullptr;
    Rect *d_rect = nullptr;
    int32_t *d_own = nullptr, *d_type = nullptr;
    int rc = 0;
    auto ok = [&](cudaError_t e) {
        if (e != cudaSuccess) rc = -1;
        return rc == 0;
    };
    auto up = [&](void *dst, const void *src, size_t bytes) {
        return bytes == 0 || ok(cudaMemcpy(dst, src, bytes, cudaMemcpyHostToDevice));
    };
    const size_t nr = rects.size(), na = c.Na;
    if (ok(cudaMalloc(&d_gli, sizeof(double) * 2 * n)) && ok(cudaMalloc(&d_ph, sizeof(double) * 2 * n)) &&
        ok(cudaMalloc(&d_occ, sizeof(double) * (na + 1))) && ok(cudaMalloc(&d_ads, sizeof(double) * (na + 1))) &&
        ok(cudaMalloc(&d_dw, sizeof(double) * (na + 1))) && ok(cudaMalloc(&d_type, sizeof(int32_t) * (na + 1))) &&
        ok(cudaMalloc(&d_cur, sizeof(double) * nc)) && ok(cudaMalloc(&d_rect, sizeof(Rect) * (nr + 1))) &&
        ok(cudaMalloc(&d_own, sizeof(int32_t) * (nr + 1))) && up(d_gli, c.gli, sizeof(double) * 2 * n) &&
        ok(cudaMemset(d_ph, 0, sizeof(double) * 2 * n)) && up(d_occ, c.occ, sizeof(double) * na) &&
        up(d_ads, c.ads, sizeof(double) * na) &&
        (c.source != RS_DT_DW || up(d_dw, c.dw, sizeof(double) * na)) &&
        up(d_type, c.type, sizeof(int32_t) * na) && (!curve || up(d_cur, c.curves, sizeof(double) * nc)) &&
        up(d_rect, rects.data(), sizeof(Rect) * nr) && up(d_own, owner.data(), sizeof(int32_t) * nr)) {
        if (nr > 0)
            rs_accumulate_kernel<<<(unsigned)nr, 256>>>(d_rect, d_own, d_occ, d_ads, d_dw, d_type,
                                                        curve ? d_cur : nullptr, c.Npoints, c.dds, c.source,
                                                        dxa, dyb, cos_gam, c.N, d_ph, d_ph + n);
        if (c.phase_grating)
            pg_apply_kernel<<<(unsigned)((n + 255) / 256), 256>>>(d_ph, d_ph + n, c.K, n, d_gli);
        else
            pot_apply_kernel<<<(unsigned)((n + 255) / 256), 256>>>(d_ph, d_ph + n, n, d_gli);
        if (ok(cudaGetLastError())) ok(cudaMemcpy(c.gli, d_gli, sizeof(double) * 2 * n, cudaMemcpyDeviceToHost));
    }
    cudaFree(d_gli);
    cudaFree(d_ph);
    cudaFree(d_occ);
    cudaFree(d_ads);
    cudaFree(d_dw);
    cudaFree(d_type);
    cudaFree(d_cur);
    cudaFree(d_rect);
    cudaFree(d_own);
    if (!rc && c.cpro) {
        if (c.periodic) {
            *c.cpro = 100.0f;                      // PG_RS.cpp:451
        } else {
            const double mpro = 100.0 / (double)c.Na;
            for (uint32_t k = 0; k < c.Na; ++k) *c.cpro += mpro;   // PG_RS.cpp:113
        }
    }
    return rc;
}

double interaction_k(double E) {
    const double lambda = cs_lambda(E);
    return lambda * sqrt(1.0 + pow((0.0242621 / lambda), 2));
}

RsCall rs_call(double a, double b, double gam, double K, double atrad, uint32_t N, uint32_t M, uint32_t Na,
               const double *xx, const double *yy, const double *dw, const double *ads, const double *occ,
               const int32_t *type, const double *curves, uint32_t Npoints, double dds, double *gli, float *cpro,
               int source, bool angstrom, bool periodic, bool phase_grating) {
    return RsCall{a, b, gam, K, atrad, N, M, Na, xx, yy, dw, ads, occ, type, curves, Npoints, dds, gli, cpro,
                  source, angstrom, periodic, phase_grating, false};
}

// ------------------------------------------------------------ reciprocal space
// Potential_rec_DT_DW (Pot_rec_DT_DW.cpp:3-134) and Potential_rec_curve_DW
// (Pot_rec_curve_DW.cpp:7-164): Fourier coefficients of the potential on the
// reflections (i Nmult, j Mmult) inside the half-grid, for the rows [SL, EL) of
// an M-row grid, added into gli (EL - SL rows of N complex doubles).
// Reflection (h, k) gets sum_atoms res(s) occ (1 + i ads) exp(-2 pi i (h x + k y)),
// res the Doyle-Turner f(s) exp(-DW s^2) / cell area, or the type's curve at s/dds.
// One thread per (i, j) pair writes its four mirrored reflections
// (+-h, +-k); atoms are grouped by species (type and, for DT, Debye-Waller
// factor) so the radial factor is evaluated once per species, and the phase
// factors come from per-atom tables built once.
struct RecArgs {
    uint32_t N, M, SL, EL, Nmult, Mmult, ni, nj, nsp;
    double A_, B_, cosg, vol, ds, dds;
    const double2 *ex, *ey;          // [atom][i], [atom][j]: exp(-2 pi i x i), exp(-2 pi i y j)
    const double *occ, *ads;         // by species-sorted atom
    const int32_t *sp_off;           // [nsp + 1]
    const int32_t *sp_type;          // [nsp]
    const double *sp_dw;             // [nsp]
    const double *curves;            // curve form; nullptr for DT
    uint32_t Npoints;
    double *gli;
};

__global__ void rec_phase_kernel(const double *coord, uint32_t na, uint32_t n, double2 *out) {
    const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (size_t)na * n) return;
    const uint32_t k = (uint32_t)(idx / n), i = (uint32_t)(idx % n);
    const double con = -2. * M_PI * coord[k] * (double)i;
    double sn, cn;
    sincos(con, &sn, &cn);
    out[idx] = make_double2(cn, sn);
}

// Radial factor of species sp: DT form at s (ss = s^2 given separately), or the
// curve at index position t; returns false where the curve ends (the reference skips).
__device__ inline bool rec_res(const RecArgs &p, int sp, double s, double ss, double t, double &res) {
    if (!p.curves) {
        res = dt_rec(c_dt, p.sp_type[sp], s) * exp(-p.sp_dw[sp] * ss) * p.vol;
        return true;
    }
    const double fl = floor(t);
    if (fl >= (double)(p.Npoints - 1)) return false;
    const uint32_t jjj = (uint32_t)fl;
    const double *c = p.curves + (size_t)p.sp_type[sp] * p.Npoints;
    res = c[jjj] + (c[jjj + 1] - c[jjj]) * (t - jjj);
    return true;
}

struct C2 {
    double re, im;
};
__device__ inline void cadd(C2 &acc, double r, double x, double y) {  // acc += r (x + i y)
    acc.re += r * x;
    acc.im += r * y;
}

__global__ void rec_kernel(RecArgs p) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t j = blockIdx.y;
    if (i >= p.ni || j >= p.nj) return;
    const long ii = (long)i * p.Nmult, jj = (long)j * p.Mmult;
    const double x = (double)i * p.A_;
    // output locations (row, column) of the up to four reflections
    bool up = false, low = false;
    if (j == 0) {
        up = p.SL == 0;
    } else {
        up = jj >= (long)p.SL && jj < (long)p.EL;
        low = (long)p.M - jj >= (long)p.SL && (long)p.M - jj < (long)p.EL;
    }
    if (!up && !low) return;
    C2 u1{0, 0}, u2{0, 0}, l1{0, 0}, l2{0, 0};
    const double y = (double)j * p.B_;
    const double y_pow2 = y * y, y_cosgam = y * p.cosg * 2.;
    for (int sp = 0; sp < (int)p.nsp; ++sp) {
        double res = 0, res1 = 0;
        if (j == 0 && i == 0) {
            // (0, 0): f(0) / area (DT) or the curve's first point
            if (p.curves) res = p.curves[(size_t)p.sp_type[sp] * p.Npoints];
            else res = dt_rec(c_dt, p.sp_type[sp], 0) * p.vol;
        } else if (j == 0) {
            const double ss = x * x * 0.25;
            if (!rec_res(p, sp, x * 0.5, ss, x * 0.5 * p.ds, res)) continue;
        } else {
            // the row's own lookup: beyond the curve the species skips the whole row
            double r0;
            if (!rec_res(p, sp, sqrt(y_pow2 * 0.25), y_pow2 * 0.25, y * p.ds * 0.5, r0)) continue;
            if (i == 0) {
                res = r0;
            } else {
                double ss = (x * x + y_pow2 + x * y_cosgam) * 0.25;
                if (!rec_res(p, sp, sqrt(ss), ss, sqrt(ss) * p.ds, res)) continue;
                ss -= x * y_cosgam * 0.5;
                if (!rec_res(p, sp, sqrt(ss), ss, sqrt(ss) * p.ds, res1)) continue;
            }
        }
        C2 s1{0, 0}, s2{0, 0}, s3{0, 0}, s4{0, 0};
        for (int k = p.sp_off[sp]; k < p.sp_off[sp + 1]; ++k) {
            const double o = p.occ[k], q = o * p.ads[k];
            const double2 e_i = i ? p.ex[(size_t)k * p.ni + i] : make_double2(1.0, 0.0);
            const double2 e_j = j ? p.ey[(size_t)k * p.nj + j] : make_double2(1.0, 0.0);
            const double cc = e_i.x * e_j.x, ss_ = e_i.y * e_j.y, cs = e_i.x * e_j.y, sc = e_i.y * e_j.x;
            // e1 = e^{i(a+b)}, e2 = e^{i(b-a)}; w = o + i q
            const double e1r = cc - ss_, e1i = cs + sc, e2r = cc + ss_, e2i = cs - sc;
            cadd(s1, 1.0, o * e1r - q * e1i, o * e1i + q * e1r);    // w e1
            cadd(s2, 1.0, o * e2r - q * e2i, o * e2i + q * e2r);    // w e2
            cadd(s3, 1.0, o * e2r + q * e2i, q * e2r - o * e2i);    // w conj(e2)
            cadd(s4, 1.0, o * e1r + q * e1i, q * e1r - o * e1i);    // w conj(e1)
        }
        cadd(u1, res, s1.re, s1.im);
        cadd(u2, res1, s2.re, s2.im);
        cadd(l1, res1, s3.re, s3.im);
        cadd(l2, res, s4.re, s4.im);
    }
    const size_t N = p.N;
    auto acc = [&](long row, long col, const C2 &v) {
        double *g = p.gli + 2 * ((size_t)(row - (long)p.SL) * N + (size_t)col);
        g[0] += v.re;
        g[1] += v.im;
    };
    if (j == 0) {
        if (i == 0) {
            acc(0, 0, u1);
        } else {                 // (i, 0) and (-i, 0): phases e^{+-ia}
            acc(0, ii, u1);
            acc(0, (long)N - ii, l2);
        }
        return;
    }
    if (i == 0) {                // (0, j) and (0, -j)
        if (up) acc(jj, 0, u1);
        if (low) acc((long)p.M - jj, 0, l2);
        return;
    }
    if (up) {
        acc(jj, ii, u1);
        acc(jj, (long)N - ii, u2);
    }
    if (low) {
        acc((long)p.M - jj, ii, l1);
        acc((long)p.M - jj, (long)N - ii, l2);
    }
}

int rec_potential(double a, double b, double gam, uint32_t Nmult, uint32_t Mmult, uint32_t N, uint32_t M,
                  uint32_t Na, uint32_t SL, uint32_t EL, const double *xx, const double *yy, const double *DW,
                  const double *ads, const double *occ, const int32_t *type, const double *curves,
                  uint32_t Npoints, double dds, double *gli, float *cpro) {
    const bool curve = curves != nullptr;
    if (!gli || N < 2 || M < 2 || Nmult == 0 || Mmult == 0 || EL <= SL || EL > M || !(a > 0) || !(b > 0))
        return -1;
    if (curve && (Npoints < 2 || !(dds > 0))) return -1;
    if (Na > 0 && (!xx || !yy || !ads || !occ || !type || (!curve && !DW))) return -1;
    if (!curve && !dt_upload()) return -1;
    // reflections i Nmult < N/2 (i >= 0) and j Mmult < M/2 (j >= 0), Pot_rec_DT_DW.cpp:29, :50
    const uint32_t ni = (N / 2 + Nmult - 1) / Nmult, nj = (M / 2 + Mmult - 1) / Mmult;
    // species: type (curve) or (type, DW) (DT); atoms sorted by species
    std::vector<uint32_t> order(Na);
    int32_t maxtype = 0;
    for (uint32_t k = 0; k < Na; ++k) {
        order[k] = k;
        if (type[k] < 0 || (!curve && type[k] >= kDTRows)) return -1;
        maxtype = type[k] > maxtype ? type[k] : maxtype;
    }
    auto key_less = [&](uint32_t p, uint32_t q) {
        if (type[p] != type[q]) return type[p] < type[q];
        if (!curve && DW[p] != DW[q]) return DW[p] < DW[q];
        return p < q;
    };
    std::sort(order.begin(), order.end(), key_less);
    std::vector<int32_t> sp_off, sp_type;
    std::vector<double> sp_dw, s_occ(Na), s_ads(Na), s_x(Na), s_y(Na);
    for (uint32_t r = 0; r < Na; ++r) {
        const uint32_t k = order[r];
        if (r == 0 || type[k] != type[order[r - 1]] || (!curve && DW[k] != DW[order[r - 1]])) {
            sp_off.push_back((int32_t)r);
            sp_type.push_back(type[k]);
            sp_dw.push_back(curve ? 0.0 : DW[k]);
        }
        s_occ[r] = occ[k];
        s_ads[r] = ads[k];
        s_x[r] = xx[k];
        s_y[r] = yy[k];
    }
    sp_off.push_back((int32_t)Na);
    const uint32_t nsp = (uint32_t)sp_type.size();
    const size_t rows = EL - SL, nout = rows * N;
    const size_t nc = curve ? (size_t)(maxtype + 1) * Npoints : 1;
    double *d_gli = nullptr, *d_occ = nullptr, *d_ads = nullptr, *d_x = nullptr, *d_y = nullptr, *d_dw = nullptr,
           *d_cur = nullptr;
    double2 *d_ex = nullptr, *d_ey = nullptr;
    int32_t *d_off = nullptr, *d_type = nullptr;
    int rc = 0;
    auto ok = [&](cudaError_t e) {
        if (e != cudaSuccess) rc = -1;
        return rc == 0;
    };
    auto up = [&](void *dst, const void *src, size_t bytes) {
        return bytes == 0 || ok(cudaMemcpy(dst, src, bytes, cudaMemcpyHostToDevice));
    };
    const size_t na1 = (size_t)Na + 1;
    if (ok(cudaMalloc(&d_gli, sizeof(double) * 2 * nout)) && ok(cudaMalloc(&d_occ, sizeof(double) * na1)) &&
        ok(cudaMalloc(&d_ads, sizeof(double) * na1)) && ok(cudaMalloc(&d_x, sizeof(double) * na1)) &&
        ok(cudaMalloc(&d_y, sizeof(double) * na1)) && ok(cudaMalloc(&d_dw, sizeof(double) * (nsp + 1))) &&
        ok(cudaMalloc(&d_cur, sizeof(double) * nc)) && ok(cudaMalloc(&d_ex, sizeof(double2) * (na1 * ni))) &&
        ok(cudaMalloc(&d_ey, sizeof(double2) * (na1 * nj))) &&
        ok(cudaMalloc(&d_off, sizeof(int32_t) * (nsp + 1))) && ok(cudaMalloc(&d_type, sizeof(int32_t) * (nsp + 1))) &&
        up(d_gli, gli, sizeof(double) * 2 * nout) && up(d_occ, s_occ.data(), sizeof(double) * Na) &&
        up(d_ads, s_ads.data(), sizeof(double) * Na) && up(d_x, s_x.data(), sizeof(double) * Na) &&
        up(d_y, s_y.data(), sizeof(double) * Na) && up(d_dw, sp_dw.data(), sizeof(double) * nsp) &&
        (!curve || up(d_cur, curves, sizeof(double) * nc)) &&
        up(d_off, sp_off.data(), sizeof(int32_t) * (nsp + 1)) && up(d_type, sp_type.data(), sizeof(int32_t) * nsp)) {
        if (Na > 0) {
            rec_phase_kernel<<<(unsigned)(((size_t)Na * ni + 255) / 256), 256>>>(d_x, Na, ni, d_ex);
            rec_phase_kernel<<<(unsigned)(((size_t)Na * nj + 255) / 256), 256>>>(d_y, Na, nj, d_ey);
        }
        RecArgs p{N, M, SL, EL, Nmult, Mmult, ni, nj, nsp, 1. / (a * sin(gam)), 1. / (b * sin(gam)), -cos(gam),
                  1. / (a * b * sin(gam)), 1.0 / dds, dds, d_ex, d_ey, d_occ, d_ads, d_off, d_type, d_dw,
                  curve ? d_cur : nullptr, Npoints, d_gli};
        if (Na > 0) rec_kernel<<<dim3((ni + 127) / 128, nj), 128>>>(p);
        if (ok(cudaGetLastError())) ok(cudaMemcpy(gli, d_gli, sizeof(double) * 2 * nout, cudaMemcpyDeviceToHost));
    }
    cudaFree(d_gli);
    cudaFree(d_occ);
    cudaFree(d_ads);
    cudaFree(d_x);
    cudaFree(d_y);
    cudaFree(d_dw);
    cudaFree(d_cur);
    cudaFree(d_ex);
    cudaFree(d_ey);
    cudaFree(d_off);
    cudaFree(d_type);
    if (!rc && cpro) {
        // 200 / M per processed row, Pot_rec_DT_DW.cpp:45, :128
        const double mpro = 200. / (double)M;
        if (SL == 0) *cpro += mpro;
        for (uint32_t j = 1; (long)j * Mmult < (long)(M / 2); ++j) {
            const long jj = (long)j * Mmult;
            const bool isup = jj >= (long)SL && jj < (long)EL;
            const bool islow = (long)M - jj >= (long)SL && (long)M - jj < (long)EL;
            if (isup || islow) *cpro += mpro;
        }
    }
    return rc;
}

}  // namespace

extern "C" {

// Propagator.cpp:5-53: gli <- exp(i (pi lambda dz s - 2 pi dz (tan tx x + tan ty y))) inside
// s < min(N/2a, M/2b)^2, 0 outside.
int CreatePropagator(double a, double b, double gam, double thickness, double E, double Xtilt,
                     double Ytilt, uint32_t N, uint32_t M, double *gli, float *cpro) {
    return propagator(a, b, gam, thickness, E, Xtilt, Ytilt, N, M, gli, cpro, 0);
}

// Propagator.cpp:55-107: gli <- gli * the same factor (0 outside).
int ApplyPropagator(double a, double b, double gam, double thickness, double E, double Xtilt,
                    double Ytilt, uint32_t N, uint32_t M, double *gli, float *cpro) {
    return propagator(a, b, gam, thickness, E, Xtilt, Ytilt, N, M, gli, cpro, 1);
}

#define MSL_RS_CURVE_ARGS                                                                                 \
    uint32_t N, uint32_t M, uint32_t Na, double *xx, double *yy, double *ads, double *occ, int32_t *type, \
        double *scatentryes, uint32_t Npoints, double dds, double *gli, float *cpro
#define MSL_RS_DTDW_ARGS                                                                                    \
    uint32_t N, uint32_t M, uint32_t Na, double *xx, double *yy, double *dw, double *ads, double *occ, \
        int32_t *type, double *gli, float *cpro
#define MSL_RS_DTTV_ARGS \
    uint32_t N, uint32_t M, uint32_t Na, double *xx, double *yy, double *ads, double *occ, int32_t *type, \
        double *gli, float *cpro

// Phase gratings, PG_RS.cpp: gli *= prod over atoms of exp(-K res occ ads) exp(-i K res occ).
int PG_rs_curve_DW_cutpot(double a, double b, double gam, double E, double atrad, MSL_RS_CURVE_ARGS) {  // :57-119
    return rs_atoms(rs_call(a, b, gam, interaction_k(E), atrad, N, M, Na, xx, yy, nullptr, ads, occ, type,
                            scatentryes, Npoints, dds, gli, cpro, RS_CURVE, false, false, true));
}
int PG_rs_curve_TV_cutpot(double a, double b, double gam, double E, double atrad, MSL_RS_CURVE_ARGS) {  // :121-186
    return rs_atoms(rs_call(a, b, gam, interaction_k(E), atrad, N, M, Na, xx, yy, nullptr, ads, occ, type,
                            scatentryes, Npoints, dds, gli, cpro, RS_CURVE, true, false, true));
}
int PG_rs_DT_DW_cutpot(double a, double b, double gam, double E, double atrad, MSL_RS_DTDW_ARGS) {  // :188-241
    return rs_atoms(rs_call(a, b, gam, interaction_k(E), atrad, N, M, Na, xx, yy, dw, ads, occ, type, nullptr, 0,
                            0.0, gli, cpro, RS_DT_DW, false, false, true));
}
int PG_rs_DT_TV_cutpot(double a, double b, double gam, double E, double atrad, MSL_RS_DTTV_ARGS) {  // :243-300
    return rs_atoms(rs_call(a, b, gam, interaction_k(E), atrad, N, M, Na, xx, yy, nullptr, ads, occ, type,
                            nullptr, 0, 0.0, gli, cpro, RS_DT_TV, true, false, true));
}
int PG_rs_curve_DW_periodic(double a, double b, double gam, double E, double atrad, MSL_RS_CURVE_ARGS) {  // :304-452
    return rs_atoms(rs_call(a, b, gam, interaction_k(E), atrad, N, M, Na, xx, yy, nullptr, ads, occ, type,
                            scatentryes, Npoints, dds, gli, cpro, RS_CURVE, false, true, true));
}
int PG_rs_DT_DW_periodic(double a, double b, double gam, double E, double atrad, MSL_RS_DTDW_ARGS) {  // :454-598
    return rs_atoms(rs_call(a, b, gam, interaction_k(E), atrad, N, M, Na, xx, yy, dw, ads, occ, type, nullptr, 0,
                            0.0, gli, cpro, RS_DT_DW, false, true, true));
}
int PG_rs_curve_TV_periodic(double a, double b, double gam, double E, double atrad, MSL_RS_CURVE_ARGS) {  // :602-751
    return rs_atoms(rs_call(a, b, gam, interaction_k(E), atrad, N, M, Na, xx, yy, nullptr, ads, occ, type,
                            scatentryes, Npoints, dds, gli, cpro, RS_CURVE, true, true, true));
}
int PG_rs_DT_TV_periodic(double a, double b, double gam, double E, double atrad, MSL_RS_DTTV_ARGS) {  // :754-897
    return rs_atoms(rs_call(a, b, gam, interaction_k(E), atrad, N, M, Na, xx, yy, nullptr, ads, occ, type,
                            nullptr, 0, 0.0, gli, cpro, RS_DT_TV, true, true, true));
}

// PG_RS.cpp:5-55: one atom over the whole grid (no box, no wrap), K given.
int PG_rs_curve_DW_cutpot_oneatom(double a, double b, double gam, double K, double atrad, uint32_t N, uint32_t M,
                                  double xx, double yy, double ads, double occ, double *scatentry,
                                  uint32_t Npoints, double dds, double *gli) {
    if (!scatentry) return -1;
    int32_t t = 0;
    RsCall c = rs_call(a, b, gam, K, atrad, N, M, 1, &xx, &yy, nullptr, &ads, &occ, &t, scatentry, Npoints, dds,
                       gli, nullptr, RS_CURVE, false, false, true);
    c.whole_grid = true;
    return rs_atoms(c);
}

// Potentials, Pot_RS.cpp: gli += sum over atoms of (res occ, res occ ads).
int Potential_rs_curve_DW_cutpot(double a, double b, double gam, double atrad, MSL_RS_CURVE_ARGS) {  // :5-55
    return rs_atoms(rs_call(a, b, gam, 1.0, atrad, N, M, Na, xx, yy, nullptr, ads, occ, type, scatentryes,
                            Npoints, dds, gli, cpro, RS_CURVE, false, false, false));
}
int Potential_rs_curve_TV_cutpot(double a, double b, double gam, double atrad, MSL_RS_CURVE_ARGS) {  // :57-109
    return rs_atoms(rs_call(a, b, gam, 1.0, atrad, N, M, Na, xx, yy, nullptr, ads, occ, type, scatentryes,
                            Npoints, dds, gli, cpro, RS_CURVE, true, false, false));
}
int Potential_rs_DT_DW_cutpot(double a, double b, double gam, double atrad, MSL_RS_DTDW_ARGS) {  // :111-155
    return rs_atoms(rs_call(a, b, gam, 1.0, atrad, N, M, Na, xx, yy, dw, ads, occ, type, nullptr, 0, 0.0, gli,
                            cpro, RS_DT_DW, false, false, false));
}
int Potential_rs_DT_TV_cutpot(double a, double b, double gam, double atrad, MSL_RS_DTTV_ARGS) {  // :157-207
    return rs_atoms(rs_call(a, b, gam, 1.0, atrad, N, M, Na, xx, yy, nullptr, ads, occ, type, nullptr, 0, 0.0,
                            gli, cpro, RS_DT_TV, true, false, false));
}
int Potential_rs_curve_DW_periodic(double a, double b, double gam, double atrad, MSL_RS_CURVE_ARGS) {  // :209-348
    return rs_atoms(rs_call(a, b, gam, 1.0, atrad, N, M, Na, xx, yy, nullptr, ads, occ, type, scatentryes,
                            Npoints, dds, gli, cpro, RS_CURVE, false, true, false));
}
int Potential_rs_DT_DW_periodic(double a, double b, double gam, double atrad, MSL_RS_DTDW_ARGS) {  // :350-486
    return rs_atoms(rs_call(a, b, gam, 1.0, atrad, N, M, Na, xx, yy, dw, ads, occ, type, nullptr, 0, 0.0, gli,
                            cpro, RS_DT_DW, false, true, false));
}
int Potential_rs_curve_TV_periodic(double a, double b, double gam, double atrad, MSL_RS_CURVE_ARGS) {  // :488-627
    return rs_atoms(rs_call(a, b, gam, 1.0, atrad, N, M, Na, xx, yy, nullptr, ads, occ, type, scatentryes,
                            Npoints, dds, gli, cpro, RS_CURVE, true, true, false));
}
int Potential_rs_DT_TV_periodic(double a, double b, double gam, double atrad, MSL_RS_DTTV_ARGS) {  // :629-763
    return rs_atoms(rs_call(a, b, gam, 1.0, atrad, N, M, Na, xx, yy, nullptr, ads, occ, type, nullptr, 0, 0.0,
                            gli, cpro, RS_DT_TV, true, true, false));
}

// Reciprocal-space potentials.
int Potential_rec_DT_DW(double a, double b, double gam, uint32_t Nmult, uint32_t Mmult, uint32_t N, uint32_t M,
                        uint32_t Na, uint32_t SL, uint32_t EL, double *xx, double *yy, double *DW, double *ads,
                        double *occ, int32_t *type, double *gli, float *cpro) {
    return rec_potential(a, b, gam, Nmult, Mmult, N, M, Na, SL, EL, xx, yy, DW, ads, occ, type, nullptr, 0, 0.0,
                         gli, cpro);
}
int Potential_rec_curve_DW(double a, double b, double gam, uint32_t Nmult, uint32_t Mmult, uint32_t N,
                           uint32_t M, uint32_t Na, uint32_t SL, uint32_t EL, double *xx, double *yy, double *ads,
                           double *occ, int32_t *type, double *scatentryes, uint32_t Npoints, double dds,
                           double *gli, float *cpro) {
    if (!scatentryes) return -1;
    return rec_potential(a, b, gam, Nmult, Mmult, N, M, Na, SL, EL, xx, yy, nullptr, ads, occ, type, scatentryes,
                         Npoints, dds, gli, cpro);
}

// Curves.cpp: Doyle-Turner scattering factors and radial curves (host code;
// these build the tables the exports above consume).
double scat_ampl_rs_DT_DW(int i, double s, double dw) {  // :12-21, s a radius
    if (i < 0 || i >= kDTRows) return 0.0;
    s *= -4.0 * M_PI * M_PI * s;
    double sf = 0;
    for (int j = 0; j < 4; ++j) {
        const double bj = h_dt[i][2 * j + 1];
        if (bj > 0) sf += h_dt[i][2 * j] / (bj + dw) * exp(s / (bj + dw));
    }
    return sf * 4 * M_PI;
}
double scat_ampl_rs2_DT_DW(int i, double s, double dw) {  // :23-32, s a squared radius
    if (i < 0 || i >= kDTRows) return 0.0;
    return dt_rs2(h_dt, i, s, dw);
}
double scat_ampl_rs2_DT_DW0(int i, double s) {  // :34-43
    if (i < 0 || i >= kDTRows) return 0.0;
    return dt_rs2(h_dt, i, s, 0.0);
}
void CreatePots_rec_DT_DW(uint32_t Ntypes, uint32_t Npoints, double dds, int32_t *types, double *DW, double _Vol,
                          double *sc) {  // :45-61
    for (uint32_t nt = 0; nt < Ntypes; ++nt) {
        double *centr = sc + (size_t)nt * Npoints;
        const int ty = types[nt];
        const double dw = DW[nt];
        double s = 0;
        for (uint32_t i = 0; i < Npoints; ++i, s += dds)
            centr[i] = (ty >= 0 && ty < kDTRows ? dt_rec(h_dt, ty, s) : 0.0) * exp(-dw * s * s) * _Vol;
    }
}
void CreatePots_rs_DT_DW(uint32_t Ntypes, uint32_t Npoints, double dds, int32_t *types, double *DW,
                         double *sc) {  // :63-81
    for (uint32_t nt = 0; nt < Ntypes; ++nt) {
        double *centr = sc + (size_t)nt * Npoints;
        double s = 0;
        for (uint32_t i = 0; i < Npoints; ++i, s += dds) centr[i] = scat_ampl_rs_DT_DW(types[nt], s, DW[nt]);
    }
}

}  // extern "C"
