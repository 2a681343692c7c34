// Register-resident Stockham line FFTs for sm_103a.
//
// One line of N complex64 values is spread over T threads; thread t holds
// x[t + T*e] for e in [0, E), E = N/T, in registers.  A plan is a sequence of
// radices R_s (each dividing E).  Stage s (span NS = R_0*...*R_{s-1}) runs
// E/R_s radix-R_s butterflies per thread on butterfly indices j = t + T*q:
// inputs x[j + r*N/R] (= register slot q + r*E/R), twiddled by
// w^(r*(j mod NS)/(NS*R)), outputs to position (j/NS)*NS*R + j mod NS + r*NS.
// Between stages the outputs go through shared memory; after the last stage
// every output lands in the register slot its input came from, so a line
// leaves the transform in natural order with the same thread ownership it
// entered with.  That is what lets the slice loop fuse pointwise work
// (transmission, propagator, band limit, detectors) between an inverse and a
// forward transform without any extra data movement.
//
// Sign: DIR = +1 computes sum_n x[n] exp(+2 pi i n k / N) (Kirkland's "fft",
// FFTW_BACKWARD), DIR = -1 the exp(-...) transform.  Neither scales.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace msl {

// ------------------------------------------------------------------ plans
// T: threads per line; radices; row_swz: shared-memory address scheme for
// contiguous lines (0: pad i + (i >> s), 1: xor i ^ ((i >> s) & 15));
// col_c: columns per column-pass tile; col_ps: row-permutation shift there.
template <int N> struct Plan;
#define MSL_PLAN(N_, T_, NST_, R0, R1, R2, R3, R4, RSWZ, RSH, CC, CPS)          \
    template <> struct Plan<N_> {                                               \
        static constexpr int N = N_, T = T_, E = N_ / T_, NSTAGE = NST_;         \
        static constexpr int row_swz = RSWZ, row_sh = RSH;                      \
        static constexpr int col_c = CC, col_ps = CPS;                          \
        static constexpr bool PK = false, PKMUL = false;                        \
        static constexpr int radix(int s) {                                     \
            return s == 0 ? R0 : s == 1 ? R1 : s == 2 ? R2 : s == 3 ? R3 : R4;  \
        }                                                                       \
    };
//       N     T   S  radices          row  sh  C   ps
MSL_PLAN(64,    8, 2,  8,  8, 1, 1, 1,  0,  3, 16, 0)
MSL_PLAN(128,  16, 3,  8,  8, 2, 1, 1,  1,  3, 16, 0)
MSL_PLAN(256,  32, 3,  8,  8, 4, 1, 1,  1,  3, 16, 0)
MSL_PLAN(512,  64, 3,  8,  8, 8, 1, 1,  1,  3,  8, 3)
MSL_PLAN(1024, 64, 3, 16,  8, 8, 1, 1,  1,  4,  8, 4)
MSL_PLAN(2048,128, 3, 16, 16, 8, 1, 1,  0,  4,  4, 4)
MSL_PLAN(384,  32, 5,  3,  4, 4, 4, 2,  0,  5, 16, 0)
MSL_PLAN(768,  64, 5,  3,  4, 4, 4, 4,  0,  5,  8, 3)
#undef MSL_PLAN

// Column-pass plan of the TMA-fed kernel: same radices (and so the same twiddle
// tables) as Plan<N>, its own threads per line T, columns per tile C, exchange
// row permutation shift PS (>= 30: none) and CTAs per SM the registers allow.
template <int N_, int T_, int C_, int PS_, int MINB_, int NBUF_ = 3> struct ColPlanT {
    using B = Plan<N_>;
    static constexpr int N = N_, T = T_, E = N_ / T_, NSTAGE = B::NSTAGE, MINB = MINB_, NBUF = NBUF_;
    static constexpr int row_swz = B::row_swz, row_sh = B::row_sh;
    static constexpr int col_c = C_, col_ps = PS_;
    static constexpr bool PK = true, PKMUL = false, OWN_TW = false;
    static constexpr int radix(int s) { return B::radix(s); }
};
// Column plans of the mixed sides with their own radices (the kernel builds the
// twiddle tables, OWN_TW): 16 (384) or 32 (768) threads per column, 8 columns
// per tile, the radix 6 / 12 stage last, exchange swizzle g(i) = i ^ ((i >> ps)
// & 1) that a CPU bank model found conflict-free for every exchange and the
// tile access.
struct ColPlanMixed384 {  // 16 threads per column, radix 8 x 8 x 6
    static constexpr int N = 384, T = 16, E = 24, NSTAGE = 3, MINB = 4, NBUF = 2;
    static constexpr int row_swz = 1, row_sh = 2, col_c = 8, col_ps = 3;
    static constexpr bool PK = true, PKMUL = false, OWN_TW = true;
    static constexpr int radix(int s) { return s < 2 ? 8 : 6; }
};
struct ColPlanMixed768 {
    static constexpr int N = 768, T = 32, E = 24, NSTAGE = 3, MINB = 2, NBUF = 2;
    static constexpr int row_swz = 1, row_sh = 3, col_c = 8, col_ps = 3;
    static constexpr bool PK = true, PKMUL = false, OWN_TW = true;
    static constexpr int radix(int s) { return s < 2 ? 8 : 12; }
};
// Tile shapes chosen by a shared-memory bank model and by timing the 512 case.
template <int N> struct ColPlan;
template <> struct ColPlan<64> : ColPlanT<64, 8, 16, 30, 4> {};
template <> struct ColPlan<128> : ColPlanT<128, 16, 16, 30, 2> {};
template <> struct ColPlan<256> : ColPlanT<256, 32, 8, 3, 2> {};
template <> struct ColPlan<384> : ColPlanMixed384 {};
template <> struct ColPlan<512> : ColPlanT<512, 32, 4, 3, 4> {};
template <> struct ColPlan<768> : ColPlanMixed768 {};
template <> struct ColPlan<1024> : ColPlanT<1024, 64, 8, 4, 1> {};
template <> struct ColPlan<2048> : ColPlanT<2048, 128, 4, 4, 1> {};

template <class P> __host__ __device__ constexpr int plan_span(int s) {
    int ns = 1;
    for (int i = 0; i < s; ++i) ns *= P::radix(i);
    return ns;
}
// Offset of stage s's twiddle table ([r][k], R_s * NS_s entries; stage 0 has none).
template <class P> __host__ __device__ constexpr int plan_tw_offset(int s) {
    int off = 0;
    for (int i = 1; i < s; ++i) off += P::radix(i) * plan_span<P>(i);
    return off;
}
template <class P> __host__ __device__ constexpr int plan_tw_size() {
    return plan_tw_offset<P>(P::NSTAGE);
}
// Shared-memory float2 slots one contiguous line needs.
template <class P> __host__ __device__ constexpr int row_line_slots() {
    return P::row_swz == 0 ? P::N + (P::N >> P::row_sh) : P::N;
}

// --------------------------------------------------------- complex helpers
// Complex add / subtract.  PK = true issues each as one packed FP32 pair
// instruction (the sm_100-family f32x2 add, round to nearest like the scalar
// form; the negation of b folds into the instruction), halving the issue slots
// of a butterfly.  Plans choose PK (the `PK` member): measured 11 % faster in the
// 512 row pass and 3-4 % in the 256 / 384 passes; the register-only passes
// (Plan<N>) keep scalar adds.
template <bool PK> __device__ __forceinline__ float2 c_add(float2 a, float2 b) {
    if constexpr (PK) return __fadd2_rn(a, b);
    else return make_float2(a.x + b.x, a.y + b.y);
}
template <bool PK> __device__ __forceinline__ float2 c_sub(float2 a, float2 b) {
    if constexpr (PK) return __fadd2_rn(a, make_float2(-b.x, -b.y));
    else return make_float2(a.x - b.x, a.y - b.y);
}
// a + DIR i u and a - DIR i u, scalar: the swapped operand needs no register pair.
template <int DIR> __device__ __forceinline__ float2 c_add_muli(float2 a, float2 u) {
    return DIR > 0 ? make_float2(a.x - u.y, a.y + u.x) : make_float2(a.x + u.y, a.y - u.x);
}
template <int DIR> __device__ __forceinline__ float2 c_sub_muli(float2 a, float2 u) {
    return DIR > 0 ? make_float2(a.x + u.y, a.y - u.x) : make_float2(a.x - u.y, a.y + u.x);
}
__device__ __forceinline__ float2 c_mul(float2 a, float2 b) {
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// Complex product by a run-time factor (a table twiddle).  PK: two packed pair
// operations, a.x (w.x, w.y) + a.y (-w.y, w.x); the operand pairs cost moves,
// so it pays only where it shortens a pass's critical path (measured: the
// half-warp column pass 7 % faster, the half-warp row pass 2 % slower).  Plans
// choose it with their `PKMUL` member.
template <bool PK> __device__ __forceinline__ float2 c_mul_rt(float2 a, float2 w) {
    if constexpr (PK)
        return __ffma2_rn(make_float2(a.y, a.y), make_float2(-w.y, w.x), __fmul2_rn(make_float2(a.x, a.x), w));
    else return c_mul(a, w);
}
__device__ __forceinline__ float2 c_scale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }
// multiply by DIR * i
template <int DIR> __device__ __forceinline__ float2 c_muli(float2 a) {
    return DIR > 0 ? make_float2(-a.y, a.x) : make_float2(a.y, -a.x);
}

// ---------------------------------------------------------- radix kernels
template <int DIR, bool PK> __device__ __forceinline__ void dft2(float2 &a, float2 &b) {
    float2 t = a;
    a = c_add<PK>(t, b);
    b = c_sub<PK>(t, b);
}

template <int DIR, bool PK> __device__ __forceinline__ void dft3(float2 &x0, float2 &x1, float2 &x2) {
    const float s3 = 0.86602540378443864676f;
    float2 t = c_add<PK>(x1, x2), u = c_sub<PK>(x1, x2);
    float2 m = make_float2(x0.x - 0.5f * t.x, x0.y - 0.5f * t.y);
    x0 = c_add<PK>(x0, t);
    float2 v = c_muli<DIR>(c_scale(u, s3));
    x1 = c_add<PK>(m, v);
    x2 = c_sub<PK>(m, v);
}

template <int DIR, bool PK>
__device__ __forceinline__ void dft4(float2 &x0, float2 &x1, float2 &x2, float2 &x3) {
    float2 t0 = c_add<PK>(x0, x2), t1 = c_sub<PK>(x0, x2);
    float2 t2 = c_add<PK>(x1, x3), u = c_sub<PK>(x1, x3);
    x0 = c_add<PK>(t0, t2);
    x2 = c_sub<PK>(t0, t2);
    x1 = c_add_muli<DIR>(t1, u);
    x3 = c_sub_muli<DIR>(t1, u);
}

template <int DIR, bool PK> __device__ __forceinline__ void dft8(float2 *a) {
    float2 e0 = a[0], e1 = a[2], e2 = a[4], e3 = a[6];
    float2 o0 = a[1], o1 = a[3], o2 = a[5], o3 = a[7];
    dft4<DIR, PK>(e0, e1, e2, e3);
    dft4<DIR, PK>(o0, o1, o2, o3);
    const float h = 0.70710678118654752440f;
    // w8^1 = (1 + DIR i) h, w8^2 = DIR i, w8^3 = (-1 + DIR i) h
    float2 t1 = make_float2(h * (o1.x - DIR * o1.y), h * (o1.y + DIR * o1.x));
    float2 t3 = make_float2(h * (-o3.x - DIR * o3.y), h * (-o3.y + DIR * o3.x));
    a[0] = c_add<PK>(e0, o0);
    a[4] = c_sub<PK>(e0, o0);
    a[1] = c_add<PK>(e1, t1);
    a[5] = c_sub<PK>(e1, t1);
    a[2] = c_add_muli<DIR>(e2, o2);
    a[6] = c_sub_muli<DIR>(e2, o2);
    a[3] = c_add<PK>(e3, t3);
    a[7] = c_sub<PK>(e3, t3);
}

// exp(DIR * i * 2 pi m / 16) for m in 0..9
template <int DIR> __device__ __forceinline__ float2 w16(int m) {
    const float c1 = 0.92387953251128675613f, s1 = 0.38268343236508977173f;
    const float h = 0.70710678118654752440f;
    float re, im;
    switch (m) {
        case 0: re = 1.f; im = 0.f; break;
        case 1: re = c1; im = s1; break;
        case 2: re = h; im = h; break;
        case 3: re = s1; im = c1; break;
        case 4: re = 0.f; im = 1.f; break;
        case 5: re = -s1; im = c1; break;
        case 6: re = -h; im = h; break;
        case 7: re = -c1; im = s1; break;
        case 8: re = -1.f; im = 0.f; break;
        default: re = -c1; im = -s1; break;  // m = 9
    }
    return make_float2(re, DIR * im);
}

template <int DIR, bool PK> __device__ __forceinline__ void dft16(float2 *a) {
    // n = 4 n1 + n2, k = k1 + 4 k2
#pragma unroll
    for (int n2 = 0; n2 < 4; ++n2) dft4<DIR, PK>(a[n2], a[4 + n2], a[8 + n2], a[12 + n2]);
    // a[4 k1 + n2] = Y[n2][k1]; twiddle by w16^(n2 k1)
#pragma unroll
    for (int k1 = 1; k1 < 4; ++k1)
#pragma unroll
        for (int n2 = 1; n2 < 4; ++n2) a[4 * k1 + n2] = c_mul(a[4 * k1 + n2], w16<DIR>(n2 * k1));
#pragma unroll
    for (int k1 = 0; k1 < 4; ++k1) dft4<DIR, PK>(a[4 * k1], a[4 * k1 + 1], a[4 * k1 + 2], a[4 * k1 + 3]);
    // X[k1 + 4 k2] sits at a[4 k1 + k2]: transpose the 4x4 block
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = i + 1; j < 4; ++j) {
            float2 t = a[4 * i + j];
            a[4 * i + j] = a[4 * j + i];
            a[4 * j + i] = t;
        }
}

// exp(DIR * i * 2 pi m / 32), m a compile-time constant after unrolling
template <int DIR> __device__ __forceinline__ float2 w32(int m) {
    const float c[9] = {1.0f, 0.98078528040323044913f, 0.92387953251128675613f, 0.83146961230254523708f,
                        0.70710678118654752440f, 0.55557023301960222474f, 0.38268343236508977173f,
                        0.19509032201612826785f, 0.0f};
    m &= 31;
    const int q = m >> 3, r = m & 7;
    const float cr = q == 0 ? c[r] : q == 1 ? -c[8 - r] : q == 2 ? -c[r] : c[8 - r];
    const float sr = q == 0 ? c[8 - r] : q == 1 ? c[r] : q == 2 ? -c[8 - r] : -c[r];
    return make_float2(cr, DIR * sr);
}

template <int DIR, bool PK> __device__ __forceinline__ void dft32(float2 *a) {
    // n = 4 n1 + n2: 8-point transforms over n1 for each n2, Y[n2][k1] at a[4 k1 + n2]
#pragma unroll
    for (int n2 = 0; n2 < 4; ++n2) {
        float2 t[8];
#pragma unroll
        for (int n1 = 0; n1 < 8; ++n1) t[n1] = a[4 * n1 + n2];
        dft8<DIR, PK>(t);
#pragma unroll
        for (int k1 = 0; k1 < 8; ++k1) a[4 * k1 + n2] = t[k1];
    }
    // twiddle by w32^(n2 k1)
#pragma unroll
    for (int k1 = 1; k1 < 8; ++k1)
#pragma unroll
        for (int n2 = 1; n2 < 4; ++n2) {
            const int m = n2 * k1;
            if (m == 8) a[4 * k1 + n2] = c_muli<DIR>(a[4 * k1 + n2]);
            else if (m == 16) a[4 * k1 + n2] = make_float2(-a[4 * k1 + n2].x, -a[4 * k1 + n2].y);
            else a[4 * k1 + n2] = c_mul(a[4 * k1 + n2], w32<DIR>(m));
        }
    // 4-point transforms over n2 for each k1: X[k1 + 8 k2] at a[4 k1 + k2]
#pragma unroll
    for (int k1 = 0; k1 < 8; ++k1) dft4<DIR, PK>(a[4 * k1], a[4 * k1 + 1], a[4 * k1 + 2], a[4 * k1 + 3]);
    float2 o[32];
#pragma unroll
    for (int k1 = 0; k1 < 8; ++k1)
#pragma unroll
        for (int k2 = 0; k2 < 4; ++k2) o[k1 + 8 * k2] = a[4 * k1 + k2];
#pragma unroll
    for (int k = 0; k < 32; ++k) a[k] = o[k];
}

// 6 = 2 x 3: n = 2 n1 + n2 (3-point transforms over n1), twiddle w6^(n2 k1),
// 2-point transforms over n2; X[k1 + 3 k2] lands in a[k1 + 3 k2].
template <int DIR, bool PK> __device__ __forceinline__ void dft6(float2 *a) {
    float2 y0[3] = {a[0], a[2], a[4]}, y1[3] = {a[1], a[3], a[5]};
    dft3<DIR, PK>(y0[0], y0[1], y0[2]);
    dft3<DIR, PK>(y1[0], y1[1], y1[2]);
    const float h = 0.5f, s3 = 0.86602540378443864676f;
    // w6^1 = (1/2, DIR s3), w6^2 = (-1/2, DIR s3)
    y1[1] = c_mul(y1[1], make_float2(h, DIR * s3));
    y1[2] = c_mul(y1[2], make_float2(-h, DIR * s3));
#pragma unroll
    for (int k1 = 0; k1 < 3; ++k1) {
        a[k1] = c_add<PK>(y0[k1], y1[k1]);
        a[k1 + 3] = c_sub<PK>(y0[k1], y1[k1]);
    }
}

// 12 = 4 x 3: n = 3 n1 + n2 (4-point transforms over n1 for each n2), twiddle
// w12^(n2 k1), 3-point transforms over n2; X[k1 + 4 k2] lands in a[k1 + 4 k2].
template <int DIR, bool PK> __device__ __forceinline__ void dft12(float2 *a) {
    float2 y[3][4];
#pragma unroll
    for (int n2 = 0; n2 < 3; ++n2) {
        y[n2][0] = a[n2];
        y[n2][1] = a[3 + n2];
        y[n2][2] = a[6 + n2];
        y[n2][3] = a[9 + n2];
        dft4<DIR, PK>(y[n2][0], y[n2][1], y[n2][2], y[n2][3]);
    }
    // w12^m for m = n2 k1: 1, 2, 3 (n2 = 1) and 2, 4, 6 (n2 = 2)
    const float c1 = 0.86602540378443864676f, h = 0.5f;
    y[1][1] = c_mul(y[1][1], make_float2(c1, DIR * h));          // w12^1
    y[1][2] = c_mul(y[1][2], make_float2(h, DIR * c1));          // w12^2
    y[1][3] = c_muli<DIR>(y[1][3]);                              // w12^3 = DIR i
    y[2][1] = c_mul(y[2][1], make_float2(h, DIR * c1));          // w12^2
    y[2][2] = c_mul(y[2][2], make_float2(-h, DIR * c1));         // w12^4
    y[2][3] = make_float2(-y[2][3].x, -y[2][3].y);               // w12^6 = -1
#pragma unroll
    for (int k1 = 0; k1 < 4; ++k1) {
        dft3<DIR, PK>(y[0][k1], y[1][k1], y[2][k1]);
        a[k1] = y[0][k1];
        a[k1 + 4] = y[1][k1];
        a[k1 + 8] = y[2][k1];
    }
}

template <int R, int DIR, bool PK> __device__ __forceinline__ void dft(float2 *a) {
    if constexpr (R == 2) dft2<DIR, PK>(a[0], a[1]);
    else if constexpr (R == 3) dft3<DIR, PK>(a[0], a[1], a[2]);
    else if constexpr (R == 4) dft4<DIR, PK>(a[0], a[1], a[2], a[3]);
    else if constexpr (R == 6) dft6<DIR, PK>(a);
    else if constexpr (R == 12) dft12<DIR, PK>(a);
    else if constexpr (R == 8) dft8<DIR, PK>(a);
    else if constexpr (R == 16) dft16<DIR, PK>(a);
    else if constexpr (R == 32) dft32<DIR, PK>(a);
    else static_assert(R == 2, "unsupported radix");
}

// ------------------------------------------------------ shared addressing
// Contiguous lines: each line owns row_line_slots<P>() float2 slots.
template <class P> struct RowAddr {
    float2 *base;
    __device__ __forceinline__ int operator()(int i) const {
        if constexpr (P::row_swz == 0) return i + (i >> P::row_sh);
        else return i ^ ((i >> P::row_sh) & 15);
    }
};
// Contiguous lines packed back to back (the TMA row tiles): always the xor
// scheme, which stays inside the line's N slots.
template <class P> struct RowXorAddr {
    float2 *base;
    __device__ __forceinline__ int operator()(int i) const { return i ^ ((i >> P::row_sh) & 15); }
};
// Contiguous lines addressed through 32-bit shared addresses.  The slot map
// f(i) = i ^ ((i >> sh) & 15) (the RowXorAddr layout) is linear over xor:
// f(a ^ b) = f(a) ^ f(b).  An exchange index splits into a thread part and a
// compile-time part with disjoint bits, i = T | K, so with the line buffer
// aligned to its own size (a power of two) the byte address of slot i is
// (base + 8 f(T)) ^ 8 f(K): one xor with an immediate per access, the
// thread parts computed once per exchange.  Same layout, same bank behaviour
// as RowXorAddr.
template <class P> struct RowXorLin {
    uint32_t base;  // shared address of the line, aligned to N * 8 bytes
    static __host__ __device__ constexpr int f(int i) { return i ^ ((i >> P::row_sh) & 15); }
};
template <class A> struct is_xor_lin { static constexpr bool value = false; };
template <class P> struct is_xor_lin<RowXorLin<P>> { static constexpr bool value = true; };

__device__ __forceinline__ void sts_f2(uint32_t addr, float2 v) {
    asm volatile("st.shared.v2.f32 [%0], {%1, %2};" ::"r"(addr), "f"(v.x), "f"(v.y) : "memory");
}
__device__ __forceinline__ float2 lds_f2(uint32_t addr) {
    float2 v;
    asm volatile("ld.shared.v2.f32 {%0, %1}, [%2];" : "=f"(v.x), "=f"(v.y) : "r"(addr) : "memory");
    return v;
}

// Column tiles: C interleaved columns, slot = perm(i) * C + c.
template <class P> struct ColAddr {
    float2 *base;
    int c;
    __device__ __forceinline__ int operator()(int i) const {
        constexpr int C = P::col_c;
        if constexpr (C >= 16 || P::col_ps >= 30) return i * C + c;
        else return (i ^ ((i >> P::col_ps) & (16 / C - 1))) * C + c;
    }
};

// Column tiles addressed through 32-bit shared addresses: slot = g(i) * C + c
// with g(i) = i ^ ((i >> ps) & M) (the ColAddr layout, M = 16/C - 1 or none).
// g is linear over xor, so for an exchange index i = T | K (thread part T,
// compile-time part K, disjoint bits) g(i) = g(T) ^ g(K).  Split g(K) into O,
// its bits inside the range of g(T) (always within the M bits), and the rest:
// g(i) = (g(T) ^ O) + (g(K) ^ O), two disjoint terms.  Each thread keeps one
// base per value of O (M + 1 of them), so every access is base + immediate.
template <class P> struct ColXorLin {
    uint32_t base;  // shared address of the tile plus 8 c
    static constexpr int C = P::col_c;
    static constexpr int M = (C >= 16 || P::col_ps >= 30) ? 0 : 16 / C - 1;
    static __host__ __device__ constexpr int g(int i) { return M ? i ^ ((i >> P::col_ps) & M) : i; }
};
template <class A> struct is_col_lin { static constexpr bool value = false; };
template <class P> struct is_col_lin<ColXorLin<P>> { static constexpr bool value = true; };

// Bits g(T) can occupy when T ranges over [0, 2^tb) shifted left by ts bits.
template <class P> __host__ __device__ constexpr int col_lin_mask(int tbits_mask) {
    return tbits_mask | ColXorLin<P>::M;
}

// ------------------------------------------------------------ the transform
// tw: this plan's stage tables (exp(+2 pi i r k / (NS R)) at [r][k]).
template <class P, int S, int DIR>
__device__ __forceinline__ void fft_stage(float2 (&v)[P::E], int t, const float2 *__restrict__ tw) {
    constexpr int R = P::radix(S), NS = plan_span<P>(S), E = P::E, Q = E / R, T = P::T;
    const float2 *tws = tw + plan_tw_offset<P>(S);
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        float2 a[R];
#pragma unroll
        for (int r = 0; r < R; ++r) a[r] = v[q + r * Q];
        if constexpr (NS > 1) {
            const int k = (t + T * q) % NS;
#pragma unroll
            for (int r = 1; r < R; ++r) {
                float2 w = tws[r * NS + k];
                if constexpr (DIR < 0) w.y = -w.y;
                a[r] = c_mul_rt<P::PKMUL>(a[r], w);
            }
        }
        dft<R, DIR, P::PK>(a);
#pragma unroll
        for (int r = 0; r < R; ++r) v[q + r * Q] = a[r];
    }
}

// The same stage with the twiddles w^r, r = 2..R-1, formed in registers from
// the table's w^1 (one shared load per distinct k instead of R - 1): w^r =
// w^(r/2) w^(r - r/2), at most three products deep.  Trades shared-memory
// bandwidth, which bounds the line transforms, for FMA work.
template <class P, int S, int DIR>
__device__ __forceinline__ void fft_stage_cw(float2 (&v)[P::E], int t, const float2 *__restrict__ tw) {
    constexpr int R = P::radix(S), NS = plan_span<P>(S), E = P::E, Q = E / R, T = P::T;
    const float2 *tws = tw + plan_tw_offset<P>(S);
    constexpr bool SHARED_K = NS > 1 && T % NS == 0;  // every q of a thread has the same k
    float2 w[R];
    auto powers = [&](int k) {
        w[1] = tws[NS + k];
        if constexpr (DIR < 0) w[1].y = -w[1].y;
#pragma unroll
        for (int r = 2; r < R; ++r) w[r] = c_mul(w[r / 2], w[r - r / 2]);
    };
    if constexpr (SHARED_K) powers(t % NS);
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        float2 a[R];
#pragma unroll
        for (int r = 0; r < R; ++r) a[r] = v[q + r * Q];
        if constexpr (NS > 1) {
            if constexpr (!SHARED_K) powers((t + T * q) % NS);
#pragma unroll
            for (int r = 1; r < R; ++r) a[r] = c_mul(a[r], w[r]);
        }
        dft<R, DIR, P::PK>(a);
#pragma unroll
        for (int r = 0; r < R; ++r) v[q + r * Q] = a[r];
    }
}

// WARP = true: the line belongs to one warp (T == 32) and the exchange needs
// only warp-level synchronisation.
template <class P, int S, bool WARP = false, class Addr>
__device__ __forceinline__ void fft_exchange(float2 (&v)[P::E], int t, const Addr &ad) {
    constexpr int R = P::radix(S), NS = plan_span<P>(S), E = P::E, Q = E / R, T = P::T;
    static_assert(!WARP || T == 32 || T == 16, "warp-owned lines: 32 threads per line, or two half-warp lines");
    if constexpr (WARP) __syncwarp(); else __syncthreads();  // previous readers are done
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        const int j = t + T * q;
        const int d = (j / NS) * NS * R + (j % NS);
#pragma unroll
        for (int r = 0; r < R; ++r) ad.base[ad(d + r * NS)] = v[q + r * Q];
    }
    if constexpr (WARP) __syncwarp(); else __syncthreads();
#pragma unroll
    for (int e = 0; e < E; ++e) v[e] = ad.base[ad(t + T * e)];
}

// The same exchange on RowXorLin addressing (warp-owned lines, power-of-two
// radices and spans).  Write index of (q, r): with j = t + T q,
// i = (j / NS) NS R + j % NS + r NS, i.e. T-part (t / NS) NS R + t % NS and
// K-part T R q + NS r when NS <= T; T-part t and K-part
// (q / (NS/T)) NS R + T (q % (NS/T)) + NS r when NS > T.  Read index t + T e.
// sync() orders the line's threads: the warp (the default) or, for lines of 64
// threads, the warp pair.
struct WarpSync {
    __device__ __forceinline__ void operator()() const { __syncwarp(); }
};
template <class P, int S, class Sync = WarpSync>
__device__ __forceinline__ void fft_exchange_xl(float2 (&v)[P::E], int t, const RowXorLin<P> &ad,
                                                const Sync &sync = Sync()) {
    constexpr int R = P::radix(S), NS = plan_span<P>(S), E = P::E, Q = E / R, T = P::T;
    static_assert((T == 64 || T == 32 || T == 16) && (NS & (NS - 1)) == 0 && (R & (R - 1)) == 0 &&
                      (P::N & (P::N - 1)) == 0,
                  "xor-linear exchange needs warp-owned (or pair-owned) lines and power-of-two radices");
    using F = RowXorLin<P>;
    const int tw_part = NS <= T ? (t / NS) * NS * R + t % NS : t;
    const uint32_t wb = ad.base + 8u * (uint32_t)F::f(tw_part);
    const uint32_t rb = ad.base + 8u * (uint32_t)F::f(t);
    sync();  // previous readers are done
#pragma unroll
    for (int q = 0; q < Q; ++q) {
#pragma unroll
        for (int r = 0; r < R; ++r) {
            const int K = NS <= T ? q * T * R + r * NS : (q / (NS / T)) * NS * R + T * (q % (NS / T)) + r * NS;
            sts_f2(wb ^ (8u * (uint32_t)F::f(K)), v[q + r * Q]);
        }
    }
    sync();
#pragma unroll
    for (int e = 0; e < E; ++e) v[e] = lds_f2(rb ^ (8u * (uint32_t)F::f(T * e)));
}

// The column exchange on ColXorLin addressing (T threads per column spread
// over the CTA, so CTA barriers; power-of-two T, radices and spans).  Index
// split as in fft_exchange_xl.
template <class P, int S>
__device__ __forceinline__ void fft_exchange_cl(float2 (&v)[P::E], int t, const ColXorLin<P> &ad) {
    constexpr int R = P::radix(S), NS = plan_span<P>(S), E = P::E, Q = E / R, T = P::T, C = P::col_c;
    static_assert((T & (T - 1)) == 0 && (NS & (NS - 1)) == 0 && (R & (R - 1)) == 0 && (P::N & (P::N - 1)) == 0,
                  "xor-linear column exchange needs power-of-two sizes");
    using G = ColXorLin<P>;
    constexpr int NB = G::M + 1;
    // write pattern: thread part and the bits it can occupy
    const int tw_part = NS <= T ? (t / NS) * NS * R + t % NS : t;
    constexpr int WMASK = col_lin_mask<P>(NS <= T ? ((T / NS - 1) * NS * R) | (NS - 1) : (T - 1));
    constexpr int RMASK = col_lin_mask<P>(T - 1);
    uint32_t wb[NB], rb[NB];
#pragma unroll
    for (int o = 0; o < NB; ++o) {
        wb[o] = ad.base + 8u * C * (uint32_t)(G::g(tw_part) ^ o);
        rb[o] = ad.base + 8u * C * (uint32_t)(G::g(t) ^ o);
    }
    __syncthreads();  // previous readers are done
#pragma unroll
    for (int q = 0; q < Q; ++q) {
#pragma unroll
        for (int r = 0; r < R; ++r) {
            const int K = NS <= T ? q * T * R + r * NS : (q / (NS / T)) * NS * R + T * (q % (NS / T)) + r * NS;
            const int gk = G::g(K), o = gk & WMASK;
            sts_f2(wb[o] + 8u * C * (uint32_t)(gk ^ o), v[q + r * Q]);
        }
    }
    __syncthreads();
#pragma unroll
    for (int e = 0; e < E; ++e) {
        const int gk = G::g(T * e), o = gk & RMASK;
        v[e] = lds_f2(rb[o] + 8u * C * (uint32_t)(gk ^ o));
    }
}

template <class P, int DIR, int S = 0, bool WARP = false, class Addr>
__device__ __forceinline__ void fft_line(float2 (&v)[P::E], int t, const Addr &ad,
                                         const float2 *__restrict__ tw) {
    if constexpr (is_xor_lin<Addr>::value) fft_stage_cw<P, S, DIR>(v, t, tw);
    else fft_stage<P, S, DIR>(v, t, tw);
    if constexpr (S + 1 < P::NSTAGE) {
        if constexpr (is_xor_lin<Addr>::value) fft_exchange_xl<P, S>(v, t, ad);
        else if constexpr (is_col_lin<Addr>::value) fft_exchange_cl<P, S>(v, t, ad);
        else fft_exchange<P, S, WARP>(v, t, ad);
        fft_line<P, DIR, S + 1, WARP>(v, t, ad, tw);
    }
}

// Two-stage plan for 512-point lines, 16 threads x 32 elements (two lines per
// warp, one per half-warp): radix 16 then radix 32, a single exchange per
// transform.  Twiddle table: stage 1 only, [r][k] = exp(+2 pi i r k / 512),
// r < 32, k < 16.
struct HalfWarpPlan512 {
    static constexpr int N = 512, T = 16, E = 32, NSTAGE = 2;
    static constexpr int row_swz = 1, row_sh = 4, col_c = 4, col_ps = 30;
    static constexpr bool PK = true, PKMUL = false, CW = false, GTW = false;
    static constexpr int GTW_OFF = 0;
    static constexpr int radix(int s) { return s == 0 ? 16 : 32; }
};
// Two-stage plan for 256-point lines, 16 threads x 16 elements (two lines per
// warp): radix 16 then radix 16, the exchange swizzle of the 512 plan.
struct HalfWarpPlan256 {
    static constexpr int N = 256, T = 16, E = 16, NSTAGE = 2;
    static constexpr int row_swz = 1, row_sh = 4, col_c = 4, col_ps = 30;
    static constexpr bool PK = true, PKMUL = false, CW = false, GTW = false;
    static constexpr int GTW_OFF = 0;
    static constexpr int radix(int) { return 16; }
};
// Two-stage plan for 1024-point lines, one warp per line (32 threads x 32
// elements): radix 32 then radix 32, a single exchange per transform.  The
// exchange swizzle i ^ ((i >> 5) & 15) keeps both of its access patterns
// (32 t + r and t + 32 e) on 16 distinct bank pairs per half-warp.
// Its 32 x 32 stage-1 table (8 KB) would cost the row kernel a CTA per SM in
// shared memory: it is read through L1 from the host-built twiddle buffer of
// side 1024 (GTW, after Plan<1024>'s tables).  Measured 70 % of HBM against
// 67 % with the powers w^r formed in registers from w^k (CW).
struct WarpPlan1024x2 {
    static constexpr int N = 1024, T = 32, E = 32, NSTAGE = 2;
    static constexpr int row_swz = 1, row_sh = 5, col_c = 4, col_ps = 30;
    static constexpr bool PK = true, PKMUL = false, CW = false, GTW = true;
    static constexpr int GTW_OFF = plan_tw_size<Plan<1024>>();
    static constexpr int radix(int) { return 32; }
};
// The same plans for the column passes: table twiddles with packed products.
struct HalfWarpColPlan512 : HalfWarpPlan512 {
    static constexpr bool PKMUL = true;
};
struct HalfWarpColPlan256 : HalfWarpPlan256 {
    static constexpr bool PKMUL = true;
};
struct WarpPairColPlan1024 : WarpPlan1024x2 {
    static constexpr bool PKMUL = true, CW = false;
};


// Stages that form twiddle powers in registers from a compact table of bases
// w^k = exp(2 pi i k / (NS R)), k < NS, stage s at offset sum_{1 <= i < s} NS_i.
template <class P> __host__ __device__ constexpr int plan_cwb_offset(int s) {
    int off = 0;
    for (int i = 1; i < s; ++i) off += plan_span<P>(i);
    return off;
}
template <class P> __host__ __device__ constexpr int plan_cwb_size() { return plan_cwb_offset<P>(P::NSTAGE); }

template <class P, int S, int DIR>
__device__ __forceinline__ void fft_stage_cwb(float2 (&v)[P::E], int t, const float2 *__restrict__ twb) {
    constexpr int R = P::radix(S), NS = plan_span<P>(S), E = P::E, Q = E / R, T = P::T;
    constexpr bool SHARED_K = NS > 1 && T % NS == 0;
    float2 w[R];
    auto powers = [&](int k) {
        w[1] = twb[plan_cwb_offset<P>(S) + k];
        if constexpr (DIR < 0) w[1].y = -w[1].y;
#pragma unroll
        for (int r = 2; r < R; ++r) w[r] = c_mul(w[r / 2], w[r - r / 2]);
    };
    if constexpr (SHARED_K) powers(t % NS);
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        float2 a[R];
#pragma unroll
        for (int r = 0; r < R; ++r) a[r] = v[q + r * Q];
        if constexpr (NS > 1) {
            if constexpr (!SHARED_K) powers((t + T * q) % NS);
#pragma unroll
            for (int r = 1; r < R; ++r) a[r] = c_mul(a[r], w[r]);
        }
        dft<R, DIR, P::PK>(a);
#pragma unroll
        for (int r = 0; r < R; ++r) v[q + r * Q] = a[r];
    }
}

// Three-stage plan for 2048-point lines owned by a warp pair (64 threads x 32
// elements): radix 16, 16, 8 with compact register twiddle powers, exchanges
// synchronised over the pair; the swizzle i ^ ((i >> 4) & 15) keeps both
// exchanges on 16 distinct bank pairs per half-warp (CPU bank model).
struct WarpPairPlan2048 {
    static constexpr int N = 2048, T = 64, E = 32, NSTAGE = 3;
    static constexpr int row_swz = 1, row_sh = 4, col_c = 4, col_ps = 30;
    static constexpr bool PK = true, PKMUL = false, CW = true;
    static constexpr int radix(int s) { return s < 2 ? 16 : 8; }
};

template <class P, int DIR, int S = 0, class Sync>
__device__ __forceinline__ void fft_line_cwb(float2 (&v)[P::E], int t, const RowXorLin<P> &ad,
                                             const float2 *__restrict__ twb, const Sync &sync) {
    fft_stage_cwb<P, S, DIR>(v, t, twb);
    if constexpr (S + 1 < P::NSTAGE) {
        fft_exchange_xl<P, S>(v, t, ad, sync);
        fft_line_cwb<P, DIR, S + 1>(v, t, ad, twb, sync);
    }
}

// Column tiles of C columns x N rows laid out by a TMA swizzle, and the exchange
// that reuses each column's own slots.
//
// ColLin64 (512-point columns, C = 8, 64-byte rows, 64-byte swizzle): element
// (r, c) at byte 64 r + (8 c ^ 16 ((r >> 1) & 3)), i.e. B(r) ^ 8 c with
// B(p) = 64 p | 16 ((p >> 1) & 3); the exchange keeps logical slot i at row
// pi(i) = i ^ ((i >> 4) & 7).  ColLin32 (1024-point columns, C = 4, 32-byte
// rows, 32-byte swizzle): B(p) = 32 p | 16 ((p >> 2) & 1), pi(i) = i ^ ((i >> 5) & 7).
// Slot i of column c is at L(i) ^ 8 c, L = B o pi.  B and pi are linear over
// xor; with the tile aligned to 32 KB (every L(i) ^ 8 c is below 32 KB) an
// access is a per-thread base xor a compile-time constant.  A column's threads
// sit in one warp (512: lane l on column l & 1 as thread l >> 1) or in a warp
// pair (1024: 16 lanes of each warp, alternating between the pair's two
// columns); either way each half-warp's sixteen 64-bit accesses cover 8 rows of
// two columns, which for the natural order (row t + T e), the exchange writes
// (T t + r) and reads (t + T e) hits sixteen distinct bank pairs: one wavefront
// per half-warp (a CPU bank model checked every pattern).
struct ColLin64 {
    static __host__ __device__ constexpr uint32_t B(uint32_t p) { return (p << 6) | (((p >> 1) & 3u) << 4); }
    static __host__ __device__ constexpr uint32_t pi(uint32_t i) { return i ^ ((i >> 4) & 7u); }
    static __host__ __device__ constexpr uint32_t L(uint32_t i) { return B(pi(i)); }
};
struct ColLin32 {
    static __host__ __device__ constexpr uint32_t B(uint32_t p) { return (p << 5) | (((p >> 2) & 1u) << 4); }
    static __host__ __device__ constexpr uint32_t pi(uint32_t i) { return i ^ ((i >> 5) & 7u); }
    static __host__ __device__ constexpr uint32_t L(uint32_t i) { return B(pi(i)); }
};

// Exchange after stage S of a column held T threads x E elements in such a tile;
// cb = tile address ^ 8 c; sync() orders the column's threads (a warp or a
// warp pair).  Index split as in fft_exchange_xl.
template <class P, int S, class Lin, class Sync>
__device__ __forceinline__ void fft_exchange_ch(float2 (&v)[P::E], int t, uint32_t cb, const Sync &sync) {
    constexpr int R = P::radix(S), NS = plan_span<P>(S), E = P::E, Q = E / R, T = P::T;
    static_assert((T == 16 || T == 32) && (NS & (NS - 1)) == 0 && (R & (R - 1)) == 0, "power-of-two column plans");
    const int tw_part = NS <= T ? (t / NS) * NS * R + t % NS : t;
    const uint32_t wb = cb ^ Lin::L((uint32_t)tw_part);
    const uint32_t rb = cb ^ Lin::L((uint32_t)t);
    sync();  // previous readers of the column are done
#pragma unroll
    for (int q = 0; q < Q; ++q) {
#pragma unroll
        for (int r = 0; r < R; ++r) {
            const int K = NS <= T ? q * T * R + r * NS : (q / (NS / T)) * NS * R + T * (q % (NS / T)) + r * NS;
            sts_f2(wb ^ Lin::L((uint32_t)K), v[q + r * Q]);
        }
    }
    sync();
#pragma unroll
    for (int e = 0; e < E; ++e) v[e] = lds_f2(rb ^ Lin::L((uint32_t)(T * e)));
}

// Warp- or half-warp-owned line with table twiddles and xor-linear exchanges.
template <class P, int DIR, int S = 0>
__device__ __forceinline__ void fft_line_tab(float2 (&v)[P::E], int t, const RowXorLin<P> &ad,
                                             const float2 *__restrict__ tw) {
    if constexpr (P::CW) fft_stage_cw<P, S, DIR>(v, t, tw);
    else fft_stage<P, S, DIR>(v, t, tw);
    if constexpr (S + 1 < P::NSTAGE) {
        fft_exchange_xl<P, S>(v, t, ad);
        fft_line_tab<P, DIR, S + 1>(v, t, ad, tw);
    }
}

// Plan with one warp per line (same radices as Plan<N>).  OWN_TW: the kernel
// builds its twiddle tables (radices differ from Plan<N>'s host tables).
template <int N_> struct WarpPlan {
    using B = Plan<N_>;
    static constexpr int N = N_, T = 32, E = N_ / 32, NSTAGE = B::NSTAGE;
    static constexpr int row_swz = B::row_swz, row_sh = B::row_sh, col_c = B::col_c, col_ps = B::col_ps;
    static constexpr bool PK = true, PKMUL = false, OWN_TW = false;
    static constexpr int radix(int s) { return B::radix(s); }
};
// The mixed sides one warp per line with fewer stages than Plan<N>, the radix
// 6 / 12 stage last so the spans before it are powers of two, and an exchange
// swizzle i ^ ((i >> sh) & 15) under which every exchange is conflict-free (a
// CPU bank model of the half-warp wavefronts checked each one): 384 = 8 x 8 x 6
// on half-warp lines (16 threads x 24 elements, two lines per warp), 768 = 8 x 8
// x 12 on warp lines (32 threads x 24 elements).
template <> struct WarpPlan<384> {  // half-warp lines (two per warp)
    static constexpr int N = 384, T = 16, E = 24, NSTAGE = 3;
    static constexpr int row_swz = 1, row_sh = 3, col_c = 4, col_ps = 30;
    static constexpr bool PK = true, PKMUL = false, OWN_TW = true;
    static constexpr int radix(int s) { return s < 2 ? 8 : 6; }
};
template <> struct WarpPlan<768> {
    static constexpr int N = 768, T = 32, E = 24, NSTAGE = 3;
    static constexpr int row_swz = 1, row_sh = 3, col_c = 4, col_ps = 30;
    static constexpr bool PK = true, PKMUL = false, OWN_TW = true;
    static constexpr int radix(int s) { return s < 2 ? 8 : 12; }
};

}  // namespace msl
