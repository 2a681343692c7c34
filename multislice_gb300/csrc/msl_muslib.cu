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

// One block per (atom, image rectangle); the rectangle of pixels and the image
// shift follow the nine periodic cases of PG_RS.cpp:333-420, or the single
// clipped case of the "cutpot" variants (PG_RS.cpp:57-119, Pot_RS.cpp:5-55),
// integer bounds by C truncation as there.  Per pixel, in FP64:
// A += res occ and B += res occ ads, with res the linear interpolation of the
// atom type's radial curve at r / dds (r beyond the curve contributes nothing).
struct Rect {
    int32_t ib, ie, jb, je;
    double x0, y0;
};

__global__ void pg_accumulate_kernel(const Rect *rects, const int32_t *atom_of, const double *occ,
                                     const double *ads, const int32_t *type, const double *curves,
                                     uint32_t Npoints, double dds, double dxa, double dyb, double cos_g,
                                     uint32_t N, double *A, double *Bacc) {
    const Rect r = rects[blockIdx.x];
    const int k = atom_of[blockIdx.x];
    const double *curk = curves + (size_t)type[k] * Npoints;
    const double o = occ[k], ad = ads[k];
    const int w = r.ie - r.ib, h = r.je - r.jb;
    if (w <= 0 || h <= 0) return;
    for (int idx = threadIdx.x; idx < w * h; idx += blockDim.x) {
        const int j = r.jb + idx / w, i = r.ib + idx % w;
        const double y = j * dyb - r.y0, x = i * dxa - r.x0;
        const double ar2 = sqrt(x * (x + 2 * y * cos_g) + y * y) / dds;
        const double fl = floor(ar2);
        if (fl >= (double)(Npoints - 1)) continue;
        const uint32_t jjj = (uint32_t)fl;
        const double rem = ar2 - jjj;
        const double res = curk[jjj] + (curk[jjj + 1] - curk[jjj]) * rem;
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

// Shared body of the curve-based real-space exports.  periodic: nine image
// rectangles, else the clipped one; phase_grating: multiply gli by the grating
// with interaction constant K, else add the potential.
int curve_rs(double a, double b, double gam, double K, double atrad, uint32_t N, uint32_t M, uint32_t Na,
             const double *xx, const double *yy, const double *ads, const double *occ, const int32_t *type,
             const double *scatentryes, uint32_t Npoints, double dds, double *gli, float *cpro, bool periodic,
             bool phase_grating);

int curve_rs(double a, double b, double gam, double K, double atrad, uint32_t N, uint32_t M, uint32_t Na,
             const double *xx, const double *yy, const double *ads, const double *occ, const int32_t *type,
             const double *scatentryes, uint32_t Npoints, double dds, double *gli, float *cpro, bool periodic,
             bool phase_grating) {
    if (cpro) *cpro = 0;
    if (!gli || N == 0 || M == 0 || Npoints < 2 || !(dds > 0)) return -1;
    if (Na > 0 && (!xx || !yy || !ads || !occ || !type || !scatentryes)) return -1;
    const double sin_gam = sin(gam), cos_gam = cos(gam);
    const double drax = atrad * sin_gam / a, dray = atrad * sin_gam / b;
    const double dxa = a / (double)N, dyb = b / (double)M;
    int32_t maxtype = 0;
    std::vector<Rect> rects;
    std::vector<int32_t> owner;
    const long LN = (long)N, LM = (long)M;
    for (uint32_t k = 0; k < Na; ++k) {
        if (type[k] < 0) return -1;
        maxtype = type[k] > maxtype ? type[k] : maxtype;
        const long ibb = (long)((xx[k] - drax) * N), iee = (long)((xx[k] + drax) * N);
        const long jbb = (long)((yy[k] - dray) * M), jee = (long)((yy[k] + dray) * M);
        const double X = xx[k] * a, Y = yy[k] * b;
        auto add = [&](long ib, long ie, long jb, long je, double x0, double y0) {
            rects.push_back({(int32_t)ib, (int32_t)ie, (int32_t)jb, (int32_t)je, x0, y0});
            owner.push_back((int32_t)k);
        };
        add(ibb > 0 ? ibb : 0, iee < LN ? iee : LN, jbb > 0 ? jbb : 0, jee < LM ? jee : LM, X, Y);
        if (!periodic) continue;
        if (jbb < 0) add(ibb > 0 ? ibb : 0, iee < LN ? iee : LN, jbb + LM, LM, X, Y + b);
        if (jee >= LM) add(ibb > 0 ? ibb : 0, iee < LN ? iee : LN, 0, jee - LM + 1, X, Y - b);
        if (ibb < 0) add(ibb + LN, LN, jbb > 0 ? jbb : 0, jee < LM ? jee : LM, X + a, Y);
        if (iee >= LN) add(0, iee - LN + 1, jbb > 0 ? jbb : 0, jee < LM ? jee : LM, X - a, Y);
        if (ibb < 0 && jbb < 0) add(ibb + LN, LN, jbb + LM, LM, X + a, Y + b);
        if (iee >= LN && jee >= LM) add(0, iee - LN + 1, 0, jee - LM + 1, X - a, Y - b);
        if (iee >= LN && jbb < 0) add(0, iee - LN + 1, jbb + LM, LM, X - a, Y + b);
        if (ibb < 0 && jee >= LM) add(ibb + LN, LN, 0, jee - LM + 1, X + a, Y - b);
    }
    const size_t n = (size_t)N * M;
    const size_t nc = (size_t)(maxtype + 1) * Npoints;
    double *d_gli = nullptr, *d_ph = nullptr, *d_occ = nullptr, *d_ads = nullptr, *d_cur = nullptr;
    Rect *d_rect = nullptr;
    int32_t *d_own = nullptr, *d_type = nullptr;
    int rc = 0;
    auto ok = [&](cudaError_t e) {
        if (e != cudaSuccess) rc = -1;
        return rc == 0;
    };
    const size_t nr = rects.size();
    if (ok(cudaMalloc(&d_gli, sizeof(double) * 2 * n)) && ok(cudaMalloc(&d_ph, sizeof(double) * 2 * n)) &&
        ok(cudaMalloc(&d_occ, sizeof(double) * (Na + 1))) && ok(cudaMalloc(&d_ads, sizeof(double) * (Na + 1))) &&
        ok(cudaMalloc(&d_type, sizeof(int32_t) * (Na + 1))) && ok(cudaMalloc(&d_cur, sizeof(double) * nc)) &&
        ok(cudaMalloc(&d_rect, sizeof(Rect) * (nr + 1))) && ok(cudaMalloc(&d_own, sizeof(int32_t) * (nr + 1))) &&
        ok(cudaMemcpy(d_gli, gli, sizeof(double) * 2 * n, cudaMemcpyHostToDevice)) &&
        ok(cudaMemset(d_ph, 0, sizeof(double) * 2 * n)) &&
        (Na == 0 || (ok(cudaMemcpy(d_occ, occ, sizeof(double) * Na, cudaMemcpyHostToDevice)) &&
                     ok(cudaMemcpy(d_ads, ads, sizeof(double) * Na, cudaMemcpyHostToDevice)) &&
                     ok(cudaMemcpy(d_type, type, sizeof(int32_t) * Na, cudaMemcpyHostToDevice)) &&
                     ok(cudaMemcpy(d_cur, scatentryes, sizeof(double) * nc, cudaMemcpyHostToDevice)) &&
                     ok(cudaMemcpy(d_rect, rects.data(), sizeof(Rect) * nr, cudaMemcpyHostToDevice)) &&
                     ok(cudaMemcpy(d_own, owner.data(), sizeof(int32_t) * nr, cudaMemcpyHostToDevice))))) {
        if (nr > 0)
            pg_accumulate_kernel<<<(unsigned)nr, 256>>>(d_rect, d_own, d_occ, d_ads, d_type, d_cur, Npoints, dds,
                                                        dxa, dyb, cos_gam, N, d_ph, d_ph + n);
        if (phase_grating)
            pg_apply_kernel<<<(unsigned)((n + 255) / 256), 256>>>(d_ph, d_ph + n, K, n, d_gli);
        else
            pot_apply_kernel<<<(unsigned)((n + 255) / 256), 256>>>(d_ph, d_ph + n, n, d_gli);
        if (ok(cudaGetLastError())) ok(cudaMemcpy(gli, d_gli, sizeof(double) * 2 * n, cudaMemcpyDeviceToHost));
    }
    cudaFree(d_gli);
    cudaFree(d_ph);
    cudaFree(d_occ);
    cudaFree(d_ads);
    cudaFree(d_type);
    cudaFree(d_cur);
    cudaFree(d_rect);
    cudaFree(d_own);
    if (!rc && cpro) *cpro = 100;
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

// PG_RS.cpp:304-446: multiply gli by the phase grating of Na atoms, each a
// tabulated radial potential curve (Npoints samples spaced dds) with absorption
// ads and occupancy occ, periodic over the cell, within atrad of the atom.
int PG_rs_curve_DW_periodic(double a, double b, double gam, double E, double atrad, uint32_t N,
                            uint32_t M, uint32_t Na, double *xx, double *yy, double *ads, double *occ,
                            int32_t *type, double *scatentryes, uint32_t Npoints, double dds,
                            double *gli, float *cpro) {
    const double lambda = cs_lambda(E);
    const double K = lambda * sqrt(1.0 + pow((0.0242621 / lambda), 2));
    return curve_rs(a, b, gam, K, atrad, N, M, Na, xx, yy, ads, occ, type, scatentryes, Npoints, dds, gli,
                    cpro, true, true);
}

// PG_RS.cpp:57-119: the same grating, each atom clipped at the cell edge.
int PG_rs_curve_DW_cutpot(double a, double b, double gam, double E, double atrad, uint32_t N, uint32_t M,
                          uint32_t Na, double *xx, double *yy, double *ads, double *occ, int32_t *type,
                          double *scatentryes, uint32_t Npoints, double dds, double *gli, float *cpro) {
    const double lambda = cs_lambda(E);
    const double K = lambda * sqrt(1.0 + pow((0.0242621 / lambda), 2));
    return curve_rs(a, b, gam, K, atrad, N, M, Na, xx, yy, ads, occ, type, scatentryes, Npoints, dds, gli,
                    cpro, false, true);
}

// Pot_RS.cpp:209-348: add the potential (real) and absorption (imaginary) of the atoms, periodic.
int Potential_rs_curve_DW_periodic(double a, double b, double gam, double atrad, uint32_t N, uint32_t M,
                                   uint32_t Na, double *xx, double *yy, double *ads, double *occ, int32_t *type,
                                   double *scatentryes, uint32_t Npoints, double dds, double *gli, float *cpro) {
    return curve_rs(a, b, gam, 1.0, atrad, N, M, Na, xx, yy, ads, occ, type, scatentryes, Npoints, dds, gli,
                    cpro, true, false);
}

// Pot_RS.cpp:5-55: the same, each atom clipped at the cell edge.
int Potential_rs_curve_DW_cutpot(double a, double b, double gam, double atrad, uint32_t N, uint32_t M,
                                 uint32_t Na, double *xx, double *yy, double *ads, double *occ, int32_t *type,
                                 double *scatentryes, uint32_t Npoints, double dds, double *gli, float *cpro) {
    return curve_rs(a, b, gam, 1.0, atrad, N, M, Na, xx, yy, ads, occ, type, scatentryes, Npoints, dds, gli,
                    cpro, false, false);
}

}  // extern "C"
