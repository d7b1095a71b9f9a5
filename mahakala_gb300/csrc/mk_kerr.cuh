// mk_kerr.cuh -- Kerr spacetime in Cartesian Kerr-Schild coordinates,
// closed-form geodesic acceleration and the RK4 step, for FP64 and FP32.
//
// The reference builds g_{mu nu} = eta + f l l (geodesics.py:88-104),
// differentiates it with jax.jacfwd and inverts it with an LU solve
// (geodesics.py:294-347).  Here the same metric is differentiated by hand:
//
//   rr = r^2 = kk + q,  kk = (x^2+y^2+z^2-a^2)/2,  q = sqrt(kk^2 + a^2 z^2)
//   d_c r = (rr x_c + a^2 z delta_c3) / (2 r q)
//   f = 2 r^3 / (r^4 + a^2 z^2),  d_c f = f (3 d_c r / r - (4 r^3 d_c r + 2 a^2 z delta_c3)/den)
//   l = (1, (r x + a y)/(rr+a^2), (r y - a x)/(rr+a^2), z/r)
//   g^{mu nu} = eta - f l^mu l^nu  with l^mu = (-1, l1, l2, l3)
//
// and with D = k^c d_c (spatial directional derivative), lv = l.k,
//   F_nu = -[Df l_nu lv + f (Dl_nu lv + l_nu Dl.k)] + 1/2 d_nu f lv^2 + f lv (d_nu l.k)
//   accel^mu = g^{mu nu} F_nu,
// which equals -Gamma^mu_ab k^a k^b, the quantity rhs() returns.  With
// F_0 = -(Df lv + f Dl.k) the spatial components read
//   F_i = l_i F_0 + f lv (d_i l.k - D l_i) + 1/2 d_i f lv^2,
// and every position derivative goes through d r: d l1 = g1 d r + (r, a, 0)
// / (rr + a^2), d l2 = g2 d r + (-a, r, 0) / (rr + a^2), d l3 = -(l3/r) d r +
// (0, 0, 1/r), so D and d_i . k need k.d r, not the nine components d_c l_i.
#pragma once

#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include <type_traits>

#include "mahakala_gb300.h"
#include "mk_dd.cuh"

namespace mk {

// cgs constants as the reference spells them (constants.py:22-31,
// electrons.py:23-29), and the products the reference evaluates in Python
// scalar arithmetic, written as the exact doubles Python produces.
constexpr double EE = 4.8032e-10;
constexpr double CL = 2.99792458e10;
constexpr double ME = 9.1094e-28;
constexpr double MP = 1.6726e-24;
constexpr double HPL = 6.6261e-27;
constexpr double C2_11_12 = 0x1.e3437e7101343p+0;      // 2.0**(11./12)
constexpr double SQRT2 = 0x1.6a09e667f3bcdp+0;         // jnp.sqrt(2)
constexpr double PI = 0x1.921fb54442d18p+1;            // np.pi
constexpr double TWO_PI_ME_CL = 0x1.8ba87a55ed610p-53; // 2.*np.pi*ME*CL
constexpr double EE2 = 0x1.105f00eff1951p-62;          // EE**2
constexpr double THREE_CL = 0x1.4f0b4f6b80000p+36;     // 3.0*CL
constexpr double ME_CL_CL = 0x1.b78aed233862dp-21;     // ME*CL*CL
constexpr double TWO_HPL = 0x1.067ca31b6f6a5p-86;      // 2.*HPL
constexpr double CL2 = 0x1.85c5de8a0455dp+69;          // CL**2
constexpr double TWO_NINTHS = 0x1.c71c71c71c71cp-3;    // 2./9.
constexpr double THIRD = 0x1.5555555555555p-2;         // 1./3
constexpr double SIXTH = 0x1.5555555555555p-3;         // 1./6 (and 1/6 in RK4)

// 1/6 in each arithmetic, built from literals so that no conversion from
// double is left to run time (a run-time double -> pair split costs FP64
// instructions in the pair code)
template <typename T>
__host__ __device__ constexpr T sixth() { return T(SIXTH); }
template <>
__host__ __device__ constexpr dd sixth<dd>() { return dd(0x1.555556p-3f, -0x1.555556p-28f); }

// exact small constants in the arithmetic code are written as float
// literals (0.5f, 2.0f, ...): the same value in double, float and pairs

// Quotient for each arithmetic: pairs divide exactly; binary64 multiplies
// by rcp64's reciprocal (within 2 ulp; the division subroutine costs the
// FP64 pipe several times more); the float (mixed-form) paths multiply by
// the hardware reciprocal (rcp.approx.ftz: ~2 ulp, two instructions
// instead of a division subroutine).
__device__ __forceinline__ float fdiv(float x, float y) { return x * rcp_ftz(y); }
__device__ __forceinline__ double fdiv(double x, double y) { return x * rcp64(y); }
__device__ __forceinline__ dd fdiv(dd x, dd y) { return x / y; }

// Kerr-Schild metric data at a point: g = eta + f l l
template <typename T>
struct KerrPoint {
    T r, f, l1, l2, l3;
};

template <typename T>
__device__ __forceinline__ KerrPoint<T> kerr_point(T x, T y, T z, T a) {
    const T aa = a * a;
    const T zz = z * z;
    const T kk = T(0.5f) * (x * x + y * y + zz - aa);
    const T rr = sqrt(kk * kk + aa * zz) + kk;
    const T r = sqrt(rr);
    KerrPoint<T> m;
    m.r = r;
    m.f = (T(2.0f) * rr * r) / (rr * rr + aa * zz);
    const T ira = T(1.0f) / (rr + aa);
    m.l1 = (r * x + a * y) * ira;
    m.l2 = (r * y - a * x) * ira;
    m.l3 = z / r;
    return m;
}

// The FP32 geodesic acceleration (mixed-precision phases): the contraction
// of the generic form below (derivatives along k from k . grad r, F_i = l_i
// F_0 + f (k.l) (d_i - D l_i) + f_i (k.l)^2 / 2), with the x and y
// components on paired FP32 instructions (two lanes of one instruction,
// each rounded as its scalar twin).  Equal to the generic form to float
// rounding.
__device__ __forceinline__ float2 pair(float u, float v) { return make_float2(u, v); }
__device__ __forceinline__ float2 both(float u) { return make_float2(u, u); }

__device__ __forceinline__ void kerr_accel_f32(float x, float y, float z, float k0, float k1, float k2, float k3,
                                               float a, float &a0, float &a1, float &a2, float &a3,
                                               KerrPoint<float> &m) {
    const float2 XY = pair(x, y), K12 = pair(k1, k2);
    const float aa = a * a;
    const float zz = z * z;
    const float kk = 0.5f * (x * x + y * y + zz - aa);
    const float Q = kk * kk + aa * zz;
    const float iq = rsqrt_ftz(Q);
    const float rr = fmaf(Q, iq, kk);        // sqrt(kk^2 + a^2 z^2) + kk
    const float ir = rsqrt_ftz(rr);
    const float r = rr * ir;
    const float i2rq = 0.5f * ir * iq;       // 1 / (2 r q)
    const float den = rr * rr + aa * zz;
    const float rra = rr + aa;
    // one division for the two reciprocals 1/den and 1/(rr + a^2)
    const float inv2 = fdiv(1.0f, den * rra);
    const float2 ID = __fmul2_rn(pair(rra, den), both(inv2));
    const float iden = ID.x, ira = ID.y;
    const float2 RXY = __fmul2_rn(both(rr * i2rq), XY);  // (dr/dx, dr/dy)
    const float rz = rra * z * i2rq;
    const float f = 2.0f * (rr * r * iden);
    const float c1 = fmaf(-2.0f, f, 3.0f * ir);  // 3/r - 4 r^3/den
    // (l1, l2) = (r x + a y, r y - a x) / (r^2 + a^2); (g1, g2) = (xy - 2 r l) / (r^2 + a^2)
    const float2 L12 = __fmul2_rn(__ffma2_rn(both(r), XY, __fmul2_rn(both(a), pair(y, -x))), both(ira));
    const float l3 = z * ir;
    const float2 G12 = __fmul2_rn(__ffma2_rn(both(-2.0f * r), L12, XY), both(ira));
    const float rira = r * ira, aira = a * ira;
    const float h = l3 * ir;
    const float Dr = k1 * RXY.x + k2 * RXY.y + k3 * rz;
    const float fc = f * c1;
    const float ft = f * (2.0f * aa * z * iden);
    const float2 FXY = __fmul2_rn(both(fc), RXY);
    const float fz = fc * rz - ft;
    const float Df = fc * Dr - ft * k3;
    const float2 U = __fmul2_rn(both(rira), K12), V = __fmul2_rn(both(aira), K12);
    const float2 DL12 = __ffma2_rn(G12, both(Dr), __fadd2_rn(U, pair(V.y, -V.x)));   // D l1, D l2
    const float Dl3 = ir * k3 - h * Dr;
    const float G = G12.x * k1 + G12.y * k2 - h * k3;
    const float2 DLXY = __ffma2_rn(RXY, both(G), __fadd2_rn(pair(U.x, V.x), pair(-V.y, U.y)));  // d_x, d_y
    const float dlz = rz * G + ir * k3;
    const float lv = k0 + L12.x * k1 + L12.y * k2 + l3 * k3;
    const float Dlv = DL12.x * k1 + DL12.y * k2 + Dl3 * k3;
    const float flv = f * lv;
    const float hl = 0.5f * lv * lv;
    const float F0 = -(Df * lv + f * Dlv);
    const float2 F12 =
        __ffma2_rn(FXY, both(hl), __ffma2_rn(both(flv), __fadd2_rn(DLXY, pair(-DL12.x, -DL12.y)), __fmul2_rn(L12, both(F0))));
    const float F3 = l3 * F0 + flv * (dlz - Dl3) + fz * hl;
    const float lF = -F0 + L12.x * F12.x + L12.y * F12.y + l3 * F3;
    const float flF = f * lF;
    const float2 A12 = __ffma2_rn(L12, both(-flF), F12);
    a0 = -F0 + flF;
    a1 = A12.x;
    a2 = A12.y;
    a3 = F3 - l3 * flF;
    m.r = r;
    m.f = f;
    m.l1 = L12.x;
    m.l2 = L12.y;
    m.l3 = l3;
}

// Geodesic acceleration dk/dlambda = -Gamma^mu_ab k^a k^b at (x, y, z).
// Also returns the metric data at the point (r, f, l), which the step rule
// and the sampler reuse.
template <typename T>
__device__ __forceinline__ void kerr_accel(T x, T y, T z, T k0, T k1, T k2, T k3, T a, T &a0, T &a1, T &a2,
                                           T &a3, KerrPoint<T> &m) {
    if constexpr (std::is_same<T, float>::value) {
        kerr_accel_f32(x, y, z, k0, k1, k2, k3, a, a0, a1, a2, a3, m);
    } else {
        // the same contraction as kerr_accel_f32 (derivatives along k from
        // k . grad r, F_i = l_i F0 + f (k.l)(d_i - D l_i) + f_i (k.l)^2/2),
        // each operation in T
        const T aa = a * a;
        const T zz = z * z;
        const T kk = T(0.5f) * (x * x + y * y + zz - aa);
        const T Q = kk * kk + aa * zz;
        const T iq = inv_sqrt(Q);
        const T rr = Q * iq + kk;                 // sqrt(kk^2 + a^2 z^2) + kk
        const T ir = inv_sqrt(rr);
        const T r = rr * ir;
        const T i2rq = T(0.5f) * ir * iq;         // 1 / (2 r q)
        const T den = rr * rr + aa * zz;
        const T rra = rr + aa;
        // one division for the two reciprocals 1/den and 1/(rr + a^2)
        const T inv2 = fdiv(T(1.0f), den * rra);
        const T iden = rra * inv2;
        const T ira = den * inv2;

        const T c = rr * i2rq;
        const T rx = c * x, ry = c * y;           // dr/dx, dr/dy
        const T rz = rra * z * i2rq;
        const T f = T(2.0f) * (rr * r * iden);
        const T c1 = T(3.0f) * ir - T(2.0f) * f;

        const T l1 = (r * x + a * y) * ira;
        const T l2 = (r * y - a * x) * ira;
        const T l3 = z * ir;
        const T tr = T(2.0f) * r;
        const T g1 = (x - tr * l1) * ira;
        const T g2 = (y - tr * l2) * ira;
        const T rira = r * ira, aira = a * ira;
        const T h = l3 * ir;

        const T Dr = k1 * rx + k2 * ry + k3 * rz;
        const T fc = f * c1;
        const T ft = f * (T(2.0f) * aa * z * iden);
        const T fx = fc * rx, fy = fc * ry, fz = fc * rz - ft;
        const T Df = fc * Dr - ft * k3;
        const T u1 = rira * k1, u2 = rira * k2, v1 = aira * k1, v2 = aira * k2;
        const T Dl1 = g1 * Dr + (u1 + v2);
        const T Dl2 = g2 * Dr + (u2 - v1);
        const T Dl3 = ir * k3 - h * Dr;
        const T G = g1 * k1 + g2 * k2 - h * k3;
        const T dlx = rx * G + (u1 - v2);
        const T dly = ry * G + (v1 + u2);
        const T dlz = rz * G + ir * k3;

        const T lv = k0 + l1 * k1 + l2 * k2 + l3 * k3;
        const T Dlv = Dl1 * k1 + Dl2 * k2 + Dl3 * k3;
        const T flv = f * lv;
        const T hl = T(0.5f) * lv * lv;
        const T F0 = -(Df * lv + f * Dlv);
        const T F1 = l1 * F0 + flv * (dlx - Dl1) + fx * hl;
        const T F2 = l2 * F0 + flv * (dly - Dl2) + fy * hl;
        const T F3 = l3 * F0 + flv * (dlz - Dl3) + fz * hl;
        const T lF = -F0 + l1 * F1 + l2 * F2 + l3 * F3;
        const T flF = f * lF;
        a0 = -F0 + flF;
        a1 = F1 - l1 * flF;
        a2 = F2 - l2 * flF;
        a3 = F3 - l3 * flF;
        m.r = r;
        m.f = f;
        m.l1 = l1;
        m.l2 = l2;
        m.l3 = l3;
    }
}

template <typename T>
__device__ __forceinline__ void kerr_accel(T x, T y, T z, T k0, T k1, T k2, T k3, T a, T &a0, T &a1, T &a2,
                                           T &a3) {
    KerrPoint<T> m;
    kerr_accel(x, y, z, k0, k1, k2, k3, a, a0, a1, a2, a3, m);
}

// RK4 step whose first-stage acceleration d1 (at s) is already known; the
// other three stages are evaluated here.  With F = (k, accel) the state's
// derivative, the stages sit at s + h F1, s + h F2 (h = dt/2) and s + dt F3
// and out = s + dt/6 (F1 + 2 F2 + 2 F3 + F4): the reference's
// k_i = dt F_i, s + k/2 and (k1 + 2k2 + 2k3 + k4)/6 (geodesics.py:317-336)
// with dt folded into the coefficients -- one fused multiply-add per
// component and stage instead of a product and a sum (the FP64 form is
// bound by its FP64 instruction count), equal to rounding.
template <typename T>
__device__ __forceinline__ void rk4_step_k1(const T s[8], const T d1[4], T dt, T a, T out[8]) {
    const T h = T(0.5f) * dt;
    T acc[8], tmp[8], d0, dd1, d2, d3;
    {
        const T F[8] = {s[4], s[5], s[6], s[7], d1[0], d1[1], d1[2], d1[3]};
#pragma unroll
        for (int i = 0; i < 8; i++) { acc[i] = F[i]; tmp[i] = s[i] + h * F[i]; }
    }
    kerr_accel(tmp[1], tmp[2], tmp[3], tmp[4], tmp[5], tmp[6], tmp[7], a, d0, dd1, d2, d3);
    {
        const T F[8] = {tmp[4], tmp[5], tmp[6], tmp[7], d0, dd1, d2, d3};
#pragma unroll
        for (int i = 0; i < 8; i++) { acc[i] = acc[i] + T(2.0f) * F[i]; tmp[i] = s[i] + h * F[i]; }
    }
    kerr_accel(tmp[1], tmp[2], tmp[3], tmp[4], tmp[5], tmp[6], tmp[7], a, d0, dd1, d2, d3);
    {
        const T F[8] = {tmp[4], tmp[5], tmp[6], tmp[7], d0, dd1, d2, d3};
#pragma unroll
        for (int i = 0; i < 8; i++) { acc[i] = acc[i] + T(2.0f) * F[i]; tmp[i] = s[i] + dt * F[i]; }
    }
    kerr_accel(tmp[1], tmp[2], tmp[3], tmp[4], tmp[5], tmp[6], tmp[7], a, d0, dd1, d2, d3);
    {
        const T F[8] = {tmp[4], tmp[5], tmp[6], tmp[7], d0, dd1, d2, d3};
        const T c = dt * sixth<T>();
#pragma unroll
        for (int i = 0; i < 8; i++) out[i] = s[i] + c * (acc[i] + F[i]);
    }
}

// RK4_gen (geodesics.py:317-336) for one ray: out = s + 1/6 (k1+2k2+2k3+k4)
template <typename T>
__device__ __forceinline__ void rk4_step(const T s[8], T dt, T a, T out[8]) {
    T d1[4];
    kerr_accel(s[1], s[2], s[3], s[4], s[5], s[6], s[7], a, d1[0], d1[1], d1[2], d1[3]);
    rk4_step_k1(s, d1, dt, a, out);
}

// ------------------------------------------------------------------------
// Float pairs (hi + lo) for the mixed form's ray state.  TwoSum is Knuth's
// error-free addition (TAOCP vol. 2, 4.2.2), FastTwoSum Dekker's (1971)
// variant for |a| >= |b|; the product error comes from one fused
// multiply-add.  No step here may be reassociated or contracted (nvcc does
// neither without fast-math; the products are explicit fmaf).
struct f2 {
    float hi, lo;
};

__device__ __forceinline__ f2 two_sum(float a, float b) {
    const float s = a + b;
    const float v = s - a;
    return {s, (a - (s - v)) + (b - v)};
}

__device__ __forceinline__ f2 fast_two_sum(float a, float b) {
    const float s = a + b;
    return {s, b - (s - a)};
}

__device__ __forceinline__ f2 f2_add(f2 x, float y) {
    f2 s = two_sum(x.hi, y);
    s.lo += x.lo;
    return fast_two_sum(s.hi, s.lo);
}

__device__ __forceinline__ f2 f2_add(f2 x, f2 y) {
    f2 s = two_sum(x.hi, y.hi);
    s.lo += x.lo + y.lo;
    return fast_two_sum(s.hi, s.lo);
}

__device__ __forceinline__ f2 f2_mul(f2 x, float b) {
    const float p = x.hi * b;
    float e = fmaf(x.hi, b, -p);
    e = fmaf(x.lo, b, e);
    return fast_two_sum(p, e);
}

__device__ __forceinline__ f2 f2_from(double d) {
    const float hi = (float)d;
    return {hi, (float)(d - (double)hi)};
}

__device__ __forceinline__ double f2_to(f2 x) { return (double)x.hi + (double)x.lo; }

// x * p for p a power of two (exact)
__host__ __device__ __forceinline__ dd dd_scale(dd x, float p) { return dd(x.hi * p, x.lo * p); }

// k^t rescaled so that g(k, k) = 0 at x, keeping the spatial wavevector:
// the root of g00 k0^2 + 2 g0i k^i k0 + gij k^i k^j = 0 nearest the current
// k0 (g00 = f - 1, g0i k^i = f l.k, gij k^i k^j = |k|^2 + f (l.k)^2 with
// l.k = l_i k^i), as the binary64 form of the FP64 queue phases solves it,
// in double-float arithmetic (~44 significant bits, all on the FP32 pipe).
// On a float-pair state the result carries no less precision than the
// state itself.  A state with no real root, or on the surface g00 = 0, is
// returned unchanged.
__host__ __device__ __forceinline__ dd renull_k0_dd(dd x, dd y, dd z, dd k0, dd k1, dd k2, dd k3, dd a) {
    const dd aa = a * a, zz = z * z;
    const dd kk = dd_scale(x * x + y * y + zz - aa, 0.5f);
    const dd Q = kk * kk + aa * zz;
    const dd rr = (Q.hi > 0.0f ? Q * inv_sqrt(Q) : dd(0.0f)) + kk;  // r^2
    const dd ir = inv_sqrt(rr);
    const dd r = rr * ir;
    const dd den = rr * rr + aa * zz, rra = rr + aa;
    const dd inv2 = dd(1.0f) / (den * rra);  // 1 / ((r^4 + a^2 z^2)(r^2 + a^2))
    const dd f = dd_scale(rr * r * (rra * inv2), 2.0f);
    const dd ira = den * inv2;  // 1 / (r^2 + a^2)
    const dd l1 = (r * x + a * y) * ira, l2 = (r * y - a * x) * ira, l3 = z * ir;
    const dd lk = l1 * k1 + l2 * k2 + l3 * k3;
    const dd A = f - dd(1.0f);
    const dd B = dd_scale(f * lk, 2.0f);
    const dd C = k1 * k1 + k2 * k2 + k3 * k3 + f * lk * lk;
    const dd disc = B * B - dd_scale(A * C, 4.0f);
    if (!(disc.hi >= 0.0f) || A.hi == 0.0f) return k0;
    const dd sq = disc.hi > 0.0f ? disc * inv_sqrt(disc) : dd(0.0f);
    const dd i2A = dd(1.0f) / dd_scale(A, 2.0f);
    const dd r1 = (sq - B) * i2A, r2 = -(B + sq) * i2A;
    return fabsf((r1 - k0).hi) < fabsf((r2 - k0).hi) ? r1 : r2;
}

// sqrt in double-float: x * (1/sqrt x); 0 at 0, NaN below
__host__ __device__ __forceinline__ dd dd_sqrt(dd x) {
    if (x.hi > 0.0f) return x * inv_sqrt(x);
    return dd(x.hi == 0.0f ? 0.0f : NAN);
}

// A grid camera's constants for the mixed forms' camera rays: the pixel
// grid coord(i) = (2i + 1) step + lo in binary64, the camera's distance
// times sin/cos of its inclination and the spin in double-float.
struct CameraDD {
    dd dsi, dci, ci, si, a;
    double step, lo;
};

__host__ __device__ __forceinline__ CameraDD camera_dd(const mk_camera &c) {
    CameraDD o;
    o.dsi = dd(c.distance * c.sin_inc);
    o.dci = dd(c.distance * c.cos_inc);
    o.ci = dd(c.cos_inc);
    o.si = dd(c.sin_inc);
    o.a = dd(c.bhspin);
    o.step = (c.fov_upper - c.fov_lower) / (double)(2 * c.pixels);
    o.lo = c.fov_lower;
    return o;
}

// the binary64 grid coordinate of grid_coord (below), rounded product then
// rounded sum, on the device or the host
__host__ __device__ __forceinline__ double grid_coord_of(int i, double step, double lo) {
#ifdef __CUDA_ARCH__
    return __dadd_rn(__dmul_rn((double)(2 * i + 1), step), lo);
#else
    volatile double t = (double)(2 * i + 1) * step;
    return t + lo;
#endif
}

// Initial state of grid-camera pixel p as float pairs, in double-float
// arithmetic (~1e-13 relative; the binary64 camera_ray below puts ~300
// instructions per ray on the FP64 pipe, 1/64 of the FP32 rate on this
// part; here only the two grid coordinates are binary64).  The image-plane
// coordinates (x, y) are the binary64 grid's (so the image centre of an odd
// grid is exactly 0 when binary64 rounds it there); the ray starts at that
// point moved to the camera (geodesics.py:121-132, 168-179): position
// (d sin i - y cos i, x, y sin i + d cos i).  Its
// direction, the cross product of the image plane's differences
// (geodesics.py:173-176), is (x^2 + y^2)(sin i, 0, cos i) exactly: every
// ray leaves the camera parallel to its line of sight (binary64 leaves
// rounding residues of ~1e-13 of the components).  k^t = 1 and the spatial
// part is rescaled to null as _Nullify does (geodesics.py:58-85, 219-230):
// the same quadratic, the same isclose rule for a vanishing discriminant,
// the same choice of root, NaN where there is no positive one (the image
// centre, x = y = 0).
__host__ __device__ __forceinline__ void camera_ray_pair(const CameraDD &c, int n, int64_t p, f2 X[4], f2 K[4]) {
    const int ix = (int)(p / n), iy = (int)(p % n);
    const dd x(grid_coord_of(ix, c.step, c.lo)), y(grid_coord_of(iy, c.step, c.lo));
    const dd x1 = c.dsi - y * c.ci, x3 = y * c.si + c.dci;
    const dd rho = x * x + y * y;
    const dd v1 = rho * c.si, v3 = rho * c.ci;
    // Kerr-Schild metric data at (x1, x, x3) (geodesics.py:88-104)
    const dd a = c.a, aa = a * a, zz = x3 * x3;
    const dd kk = dd_scale(x1 * x1 + x * x + zz - aa, 0.5f);
    const dd rr = dd_sqrt(kk * kk + aa * zz) + kk;
    const dd r = dd_sqrt(rr);
    const dd f = dd_scale(rr * r, 2.0f) / (rr * rr + aa * zz);
    const dd l1 = (r * x1 + a * x) / (rr + aa), l3 = x3 / r;
    // g(v, v) = A (k^t)^2 + 2 b k^t + C for v = (k^t, v1, 0, v3)
    const dd lv = l1 * v1 + l3 * v3;
    const dd A = f - dd(1.0f), b = f * lv, C = v1 * v1 + v3 * v3 + f * lv * lv;
    const dd bb = b * b, AC = A * C, disc = bb - AC;
    const bool close = fabsf(disc.hi) <= 1e-8f + 1e-5f * fabsf(AC.hi);
    const dd sq = close ? dd(0.0f) : dd_sqrt(disc);
    const dd D = -(b.hi < 0.0f ? b : b + sq);
    const dd q1 = D / A, q2 = C / D;
    dd S = dd(NAN);
    if (!(q1.hi != q1.hi) && !(q2.hi != q2.hi)) {
        const bool lt = q1.hi < q2.hi || (q1.hi == q2.hi && q1.lo < q2.lo);
        const dd d1 = lt ? q1 : q2, d2 = lt ? q2 : q1;
        if (d1.hi > 0.0f) S = d1;
        else if (d2.hi > 0.0f) S = d2;
    }
    const dd k1 = v1 / S, k3 = v3 / S;
    X[0] = {0.0f, 0.0f};
    X[1] = {x1.hi, x1.lo};
    X[2] = {x.hi, x.lo};
    X[3] = {x3.hi, x3.lo};
    K[0] = {1.0f, 0.0f};
    K[1] = {k1.hi, k1.lo};
    K[2] = {0.0f, 0.0f};
    K[3] = {k3.hi, k3.lo};
}

// The same operations on two components at once (float2 lanes), on paired
// FP32 instructions; every lane rounds exactly as the scalar steps above
// (x - y is formed as fma(y, -1, x), -p as the product with -b).
struct f2v {
    float2 hi, lo;
};

__device__ __forceinline__ f2v f2v_of(f2 u, f2 v) { return {pair(u.hi, v.hi), pair(u.lo, v.lo)}; }
__device__ __forceinline__ f2 f2v_x(f2v p) { return {p.hi.x, p.lo.x}; }
__device__ __forceinline__ f2 f2v_y(f2v p) { return {p.hi.y, p.lo.y}; }
__device__ __forceinline__ float2 sub2(float2 x, float2 y) { return __ffma2_rn(y, both(-1.0f), x); }

__device__ __forceinline__ f2v two_sum2(float2 a, float2 b) {
    const float2 s = __fadd2_rn(a, b);
    const float2 v = sub2(s, a);
    return {s, __fadd2_rn(sub2(a, sub2(s, v)), sub2(b, v))};
}

__device__ __forceinline__ f2v fast_two_sum2(float2 a, float2 b) {
    const float2 s = __fadd2_rn(a, b);
    return {s, sub2(b, sub2(s, a))};
}

__device__ __forceinline__ f2v f2v_add(f2v x, float2 y) {
    f2v s = two_sum2(x.hi, y);
    s.lo = __fadd2_rn(s.lo, x.lo);
    return fast_two_sum2(s.hi, s.lo);
}

__device__ __forceinline__ f2v f2v_add(f2v x, f2v y) {
    f2v s = two_sum2(x.hi, y.hi);
    s.lo = __fadd2_rn(s.lo, __fadd2_rn(x.lo, y.lo));
    return fast_two_sum2(s.hi, s.lo);
}

__device__ __forceinline__ f2v f2v_mul(f2v x, float b) {
    const float2 p = __fmul2_rn(x.hi, both(b));
    float2 e = __ffma2_rn(x.hi, both(b), __fmul2_rn(x.hi, both(-b)));
    e = __ffma2_rn(x.lo, both(b), e);
    return fast_two_sum2(p, e);
}

// The float-pair state update of one RK4 step: X += dt K + dXa, K += dK,
// components 1-2 and (of K) 0-3 in pairs.  The time coordinate
// X[0] is not advanced: nothing on the imaging path reads it (the sampler
// and the step rule use the metric at x^1..x^3 and k), so the float phases
// leave it at its value from the camera.
__device__ __forceinline__ void pair_state_update(const f2 X[4], const f2 K[4], float dt, const float dXa[4],
                                                  const float dK[4], f2 Xo[4], f2 Ko[4]) {
    const f2v x12 = f2v_add(f2v_of(X[1], X[2]), f2v_add(f2v_mul(f2v_of(K[1], K[2]), dt), pair(dXa[1], dXa[2])));
    Xo[0] = X[0];
    Xo[1] = f2v_x(x12);
    Xo[2] = f2v_y(x12);
    Xo[3] = f2_add(X[3], f2_add(f2_mul(K[3], dt), dXa[3]));
    const f2v k12 = f2v_add(f2v_of(K[1], K[2]), pair(dK[1], dK[2]));
    const f2v k03 = f2v_add(f2v_of(K[0], K[3]), pair(dK[0], dK[3]));
    Ko[0] = f2v_x(k03);
    Ko[1] = f2v_x(k12);
    Ko[2] = f2v_y(k12);
    Ko[3] = f2v_y(k03);
}

// The three inner stages and the combination of one RK4 step in float
// (RK4_gen, geodesics.py:317-336, written for x'' = a(x, x')): x, k the
// state in float, a1 the acceleration there.  Returns dXa = dt^2/6 (a1 + a2
// + a3) (the position increment is dt k + dXa; the caller forms dt k in its
// own precision) and dK = dt/6 (a1 + 2 a2 + 2 a3 + a4).  Components 1-2 and
// 0-3 go in pairs through paired FP32 instructions, each lane formed as
// the scalar fma(h, k, x) chain.
__device__ __forceinline__ void rk4_stages_f32(const float x[4], const float k[4], const float a1[4], float dt,
                                               float a, float dXa[4], float dK[4]) {
    const float h = 0.5f * dt;
    const float2 H = both(h), DT = both(dt);
    const float2 x12 = pair(x[1], x[2]), k12 = pair(k[1], k[2]), k03 = pair(k[0], k[3]);
    const float2 a1_12 = pair(a1[1], a1[2]), a1_03 = pair(a1[0], a1[3]);
    float a2[4], a3[4], a4[4];
    // stage 2 at (x + h k, k + h a1)
    const float2 s12 = __ffma2_rn(H, a1_12, k12), s03 = __ffma2_rn(H, a1_03, k03);
    float2 p12 = __ffma2_rn(H, k12, x12);
    kerr_accel(p12.x, p12.y, fmaf(h, k[3], x[3]), s03.x, s12.x, s12.y, s03.y, a, a2[0], a2[1], a2[2], a2[3]);
    // stage 3 at (x + h (k + h a1), k + h a2)
    const float2 a2_12 = pair(a2[1], a2[2]), a2_03 = pair(a2[0], a2[3]);
    const float2 u12 = __ffma2_rn(H, a2_12, k12), u03 = __ffma2_rn(H, a2_03, k03);
    p12 = __ffma2_rn(H, s12, x12);
    kerr_accel(p12.x, p12.y, fmaf(h, s03.y, x[3]), u03.x, u12.x, u12.y, u03.y, a, a3[0], a3[1], a3[2], a3[3]);
    // stage 4 at (x + dt (k + h a2), k + dt a3)
    const float2 a3_12 = pair(a3[1], a3[2]), a3_03 = pair(a3[0], a3[3]);
    const float2 w12 = __ffma2_rn(DT, a3_12, k12), w03 = __ffma2_rn(DT, a3_03, k03);
    p12 = __ffma2_rn(DT, u12, x12);
    kerr_accel(p12.x, p12.y, fmaf(dt, u03.y, x[3]), w03.x, w12.x, w12.y, w03.y, a, a4[0], a4[1], a4[2], a4[3]);
    const float c = dt * dt * (1.0f / 6.0f);
    const float d = dt * (1.0f / 6.0f);
    const float2 C = both(c), D = both(d), TWO = both(2.0f);
    const float2 a4_12 = pair(a4[1], a4[2]), a4_03 = pair(a4[0], a4[3]);
    const float2 x_12 = __fmul2_rn(C, __fadd2_rn(__fadd2_rn(a1_12, a2_12), a3_12));
    const float2 k_12 = __fmul2_rn(D, __fadd2_rn(__ffma2_rn(TWO, a3_12, __ffma2_rn(TWO, a2_12, a1_12)), a4_12));
    const float2 k_03 = __fmul2_rn(D, __fadd2_rn(__ffma2_rn(TWO, a3_03, __ffma2_rn(TWO, a2_03, a1_03)), a4_03));
    dXa[0] = 0.0f;  // the time coordinate is not advanced (pair_state_update)
    dXa[1] = x_12.x;
    dXa[2] = x_12.y;
    dXa[3] = c * (a1[3] + a2[3] + a3[3]);
    dK[0] = k_03.x;
    dK[1] = k_12.x;
    dK[2] = k_12.y;
    dK[3] = k_03.y;
}

// RK4 on a float-pair state (X = x^mu, K = k^mu), accelerations in float.
// The position increment of RK4 is dt k + dt^2/6 (a1 + a2 + a3); its
// leading term is formed in pair precision, so neither rounding of the
// position (ulp(1000) = 6e-5 in float) nor of the direction accumulates
// along the 1000 M approach from the camera.  a1 = acceleration at X, K.
__device__ __forceinline__ void rk4_step_pair(const f2 X[4], const f2 K[4], const float a1[4], float dt, float a,
                                              f2 Xo[4], f2 Ko[4]) {
    float x[4], k[4], dXa[4], dK[4];
#pragma unroll
    for (int i = 0; i < 4; i++) { x[i] = X[i].hi; k[i] = K[i].hi; }
    rk4_stages_f32(x, k, a1, dt, a, dXa, dK);
    pair_state_update(X, K, dt, dXa, dK, Xo, Ko);
}

// The RK4 increments of one step in float, for a state held elsewhere in
// higher precision: x, k the state rounded to float, a1 the acceleration
// there (rk4_stages_f32).
__device__ __forceinline__ void rk4_increment_f32(const float x[4], const float k[4], const float a1[4], float dt,
                                                  float a, float dXa[4], float dK[4]) {
    rk4_stages_f32(x, k, a1, dt, a, dXa, dK);
}

// radius_cal (geodesics.py:284-291): the KS radius the step rule uses
template <typename T>
__device__ __forceinline__ T radius_cal(T x, T y, T z, T a) {
    const T R = sqrt(x * x + y * y + z * z);
    const T q = R * R - a * a;
    return sqrt((q + sqrt(q * q + T(4) * (a * a) * (z * z))) / T(2));
}

__host__ __device__ __forceinline__ double radius_eh(double a) { return 1.0 + sqrt(1.0 - a * a); }

// dt rule of geodesic_step (geodesics.py:249-252); why = stop reason
template <typename T>
__device__ __forceinline__ T reference_dt(T r, T r_eh, T div, T tol, int &why) {
    const T dt = -fdiv(r - r_eh, div);
    why = MK_RAY_ACTIVE;
    if (isnan(dt)) { why = MK_RAY_NAN; return T(0); }
    const T adiv = fabs(dt) * div;
    if (adiv < tol) { why = MK_RAY_CAPTURED; return T(0); }
    if (adiv > T(1500)) { why = MK_RAY_ESCAPED; return T(0); }
    return dt;
}

// ------------------------------------------------------------- camera
// _Image_to_BH (geodesics.py:204-209)
__device__ __forceinline__ void image_to_bh(double x, double y, double z, double ci, double si,
                                            double d, double o[3]) {
    o[0] = __dadd_rn(__dadd_rn(__dmul_rn(-y, ci), __dmul_rn(z, si)), __dmul_rn(d, si));
    o[1] = x;
    o[2] = __dadd_rn(__dadd_rn(__dmul_rn(y, si), __dmul_rn(z, ci)), __dmul_rn(d, ci));
}

// _Nullify with p=1 (geodesics.py:58-85): rescales v[1..3] so g(v,v) = 0
__device__ __forceinline__ void nullify(const double x[4], double a, double v[4]) {
    const KerrPoint<double> m = kerr_point(x[1], x[2], x[3], a);
    const double l[4] = {1.0, m.l1, m.l2, m.l3};
    double g[4][4];
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 4; j++)
            g[i][j] = __dadd_rn((i == j) ? (i == 0 ? -1.0 : 1.0) : 0.0, __dmul_rn(m.f, __dmul_rn(l[i], l[j])));
    const double A = __dmul_rn(__dmul_rn(v[0], g[0][0]), v[0]);
    const double b = __dmul_rn(__dadd_rn(__dadd_rn(__dmul_rn(v[1], g[1][0]), __dmul_rn(v[2], g[2][0])),
                                         __dmul_rn(v[3], g[3][0])), v[0]);
    double w[3];
#pragma unroll
    for (int j = 0; j < 3; j++)
        w[j] = __dadd_rn(__dadd_rn(__dmul_rn(v[1], g[1][1 + j]), __dmul_rn(v[2], g[2][1 + j])),
                         __dmul_rn(v[3], g[3][1 + j]));
    const double C = __dadd_rn(__dadd_rn(__dmul_rn(w[0], v[1]), __dmul_rn(w[1], v[2])), __dmul_rn(w[2], v[3]));
    const double bb = __dmul_rn(b, b), AC = __dmul_rn(A, C);
    const bool close = fabs(bb - AC) <= (1e-8 + 1e-5 * fabs(AC));
    const double dd = close ? 0.0 : bb - AC;
    const double bs = (b < 0.0) ? 0.0 : 1.0;  // heaviside(b, 1)
    const double D = -(b + bs * sqrt(dd));
    const double x1 = D / A, x2 = C / D;
    double d1, d2;
    if (isnan(x1) || isnan(x2)) { d1 = d2 = nan(""); }
    else { d1 = fmin(x1, x2); d2 = fmax(x1, x2); }
    const double S = (d1 > 0.0) ? d1 : ((d2 > 0.0) ? d2 : nan(""));
    v[1] = v[1] / S;
    v[2] = v[2] / S;
    v[3] = v[3] / S;
}

// grid pixel centre: np.linspace(lo, hi, 2n+1)[1::2][i] = (2i+1)*step + lo
__device__ __forceinline__ double grid_coord(int i, int n, double lo, double hi) {
    const double step = (hi - lo) / (double)(2 * n);
    return __dadd_rn(__dmul_rn((double)(2 * i + 1), step), lo);
}

// jnp.linspace(lo, hi, 2n+1)[1::2][i] (equator camera, geodesics.py:185):
// lo*(1 - t) + hi*t with t = (2i+1)/(2n)
__device__ __forceinline__ double jnp_grid_coord(int i, int n, double lo, double hi) {
    const double t = (double)(2 * i + 1) / (double)(2 * n);
    return __dadd_rn(__dmul_rn(lo, 1.0 - t), __dmul_rn(hi, t));
}

// one camera pixel at image-plane (x, y) (geodesics.py:168-179, 121-132)
__device__ __forceinline__ void camera_pixel(double x, double y, double ci, double si, double d,
                                             double a, double s[8]) {
    double org[3], ini[3], per[3];
    image_to_bh(0.0, 0.0, 0.0, ci, si, d, org);
    image_to_bh(x, y, 0.0, ci, si, d, ini);
    image_to_bh(__dadd_rn(x, y), __dsub_rn(y, x), 0.0, ci, si, d, per);
    double v1[3], v2[3];
#pragma unroll
    for (int i = 0; i < 3; i++) { v1[i] = __dadd_rn(-ini[i], org[i]); v2[i] = __dsub_rn(per[i], ini[i]); }
    s[0] = 0.0;
    s[1] = ini[0];
    s[2] = ini[1];
    s[3] = ini[2];
    double v[4];
    v[0] = 1.0;
    v[1] = __dsub_rn(__dmul_rn(v1[1], v2[2]), __dmul_rn(v1[2], v2[1]));
    v[2] = __dsub_rn(__dmul_rn(v1[2], v2[0]), __dmul_rn(v1[0], v2[2]));
    v[3] = __dsub_rn(__dmul_rn(v1[0], v2[1]), __dmul_rn(v1[1], v2[0]));
    nullify(s, a, v);
    s[4] = v[0];
    s[5] = v[1];
    s[6] = v[2];
    s[7] = v[3];
}

// initial state of pixel p of a camera
__device__ __forceinline__ void camera_ray(const mk_camera &c, int64_t p, double s[8]) {
    const int n = c.pixels;
    if (c.kind == MK_CAMERA_EQUATOR) {
        double x[4] = {0.0, c.distance, jnp_grid_coord((int)p, n, c.fov_lower, c.fov_upper), 0.0};
        double v[4] = {1.0, 1.0, 0.0, 0.0};
        nullify(x, c.bhspin, v);
        s[0] = x[0]; s[1] = x[1]; s[2] = x[2]; s[3] = x[3];
        s[4] = v[0]; s[5] = v[1]; s[6] = v[2]; s[7] = v[3];
        return;
    }
    const int ix = (int)(p / n), iy = (int)(p % n);
    camera_pixel(grid_coord(ix, n, c.fov_lower, c.fov_upper), grid_coord(iy, n, c.fov_lower, c.fov_upper),
                 c.cos_inc, c.sin_inc, c.distance, c.bhspin, s);
}

// initial state of pixel p as float pairs, for the mixed forms: grid
// cameras in double-float (camera_ray_pair), equator cameras in binary64
__device__ __forceinline__ void camera_pair(const mk_camera &c, int64_t p, f2 X[4], f2 K[4]) {
    if (c.kind == MK_CAMERA_GRID) {
        camera_ray_pair(camera_dd(c), c.pixels, p, X, K);
        return;
    }
    double s[8];
    camera_ray(c, p, s);
#pragma unroll
    for (int i = 0; i < 4; i++) {
        X[i] = f2_from(s[i]);
        K[i] = f2_from(s[4 + i]);
    }
}

}  // namespace mk
