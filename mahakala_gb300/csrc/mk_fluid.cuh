// mk_fluid.cuh -- GRMHD snapshot sampling, fluid frame, electron
// temperature and thermal synchrotron coefficients (device functions).
//
// Snapshot layout in HBM: meshblocks with one ghost layer, AoS float32,
// [mb][k][j][i][prim] with prim = dens, velx, vely, velz, eint, bcc1..3.
// One cell is 32 bytes (one DRAM sector); the two x-neighbours a trilinear
// corner pair needs are 64 contiguous bytes.
#pragma once

#include "mk_kerr.cuh"

namespace mk {

// ------------------------------------------------------------- lookup
// The block with left < x <= right on all three axes, the last such block
// when several are (athenak.py:657-670 scans them all), -1 for none.  The
// finest-level table gives the candidate; the exact face test decides, and
// a point within rounding of the candidate's faces is moved one table cell
// across them until the test holds.  Blocks that tile the domain leave at
// most one block passing; where two do (faces an ulp apart) the higher
// index wins, as in the scan.
__device__ __forceinline__ bool in_block(const double *__restrict__ f, double x, double y, double z) {
    return x > __ldg(f) && x <= __ldg(f + 1) && y > __ldg(f + 2) && y <= __ldg(f + 3) && z > __ldg(f + 4) &&
           z <= __ldg(f + 5);
}

__device__ __forceinline__ int table_at(const mk_snapshot_view &s, const int c[3]) {
    if (c[0] < 0 || c[1] < 0 || c[2] < 0 || c[0] >= s.nb[0] || c[1] >= s.nb[1] || c[2] >= s.nb[2]) return -1;
    return __ldg(s.table + ((int64_t)c[2] * s.nb[1] + c[1]) * s.nb[0] + c[0]);
}

__device__ __forceinline__ int find_block(const mk_snapshot_view &s, double x, double y, double z) {
    const double xs[3] = {x, y, z};
    int c[3];
#pragma unroll
    for (int a = 0; a < 3; a++) {
        // candidate table cell (the face tests below decide exactly)
        const double u = floor((xs[a] - s.lo[a]) * rcp64(s.width[a]));
        if (!(u >= -1.0 && u <= (double)s.nb[a])) return -1;  // far outside (or NaN)
        c[a] = (int)u < 0 ? 0 : ((int)u >= s.nb[a] ? s.nb[a] - 1 : (int)u);
    }
    int mb = -1;
    for (int it = 0; it < 4; ++it) {
        mb = table_at(s, c);
        if (mb < 0) return -1;
        const double *f = s.faces + 6 * (int64_t)mb;
        bool moved = false;
#pragma unroll
        for (int a = 0; a < 3; a++) {
            if (xs[a] <= __ldg(f + 2 * a)) { --c[a]; moved = true; }
            else if (xs[a] > __ldg(f + 2 * a + 1)) { ++c[a]; moved = true; }
        }
        if (!moved) break;
        if (it == 3) return -1;
    }
    if (mb < 0) return -1;
    // neighbours across a face the point lies on (to rounding) that also
    // pass the test: the scan keeps the last
    const double *f = s.faces + 6 * (int64_t)mb;
    int lo_[3], hi_[3];
#pragma unroll
    for (int a = 0; a < 3; a++) {
        const double w = __ldg(f + 2 * a + 1) - __ldg(f + 2 * a);
        lo_[a] = xs[a] - __ldg(f + 2 * a) <= 1e-12 * w ? -1 : 0;
        hi_[a] = __ldg(f + 2 * a + 1) - xs[a] <= 1e-12 * w ? 1 : 0;
    }
    if (lo_[0] | hi_[0] | lo_[1] | hi_[1] | lo_[2] | hi_[2]) {
        for (int dk = lo_[2]; dk <= hi_[2]; dk++)
            for (int dj = lo_[1]; dj <= hi_[1]; dj++)
                for (int di = lo_[0]; di <= hi_[0]; di++) {
                    const int cc[3] = {c[0] + di, c[1] + dj, c[2] + dk};
                    const int o = table_at(s, cc);
                    if (o > mb && in_block(s.faces + 6 * (int64_t)o, x, y, z)) mb = o;
                }
    }
    return mb;
}

// float floor_divide / remainder with NumPy (= jnp) semantics
__device__ __forceinline__ double py_floordiv(double x, double y) {
    const double mod = fmod(x, y);
    double div = (x - mod) / y;
    if (mod != 0.0 && ((y < 0.0) != (mod < 0.0))) div -= 1.0;
    if (div != 0.0) {
        double fl = floor(div);
        if (div - fl > 0.5) fl += 1.0;
        return fl;
    }
    return copysign(0.0, x / y);
}
__device__ __forceinline__ double py_mod1(double x) {
    double m = fmod(x, 1.0);
    if (m != 0.0 && m < 0.0) m += 1.0;
    return m;
}

// ghost-shifted cell index and offset (athenak.py:718-733)
struct CellPos {
    int mb;
    int idx[3];
    double del[3];
};

__device__ __forceinline__ bool locate(const mk_snapshot_view &s, double x, double y, double z, CellPos &c) {
    const int mb = find_block(s, x, y, z);
    if (mb < 0) return false;
    c.mb = mb;
    const double *g = s.geom + 6 * (int64_t)mb;
    const double xs[3] = {x, y, z};
#pragma unroll
    for (int a = 0; a < 3; a++) {
        const double d = __ldg(g + 3 + a);
        const double t = xs[a] - __ldg(g + a) + d;
        c.del[a] = py_mod1(t / d);
        int i = (int)py_floordiv(t, d);
        // the face test above guarantees 0 <= i <= n; clamp keeps loads in bounds
        c.idx[a] = i < 0 ? 0 : (i > s.n ? s.n : i);
    }
    return true;
}

// locate for the fused FP64 render: the same block (find_block), the cell
// index and offset from q = t / d taken as t * rcp64(d) and split by floor.
// Where that differs from the reference's quotient (by an ulp, at a cell
// edge) it picks the neighbouring cell with the offset at the other end,
// and trilinear interpolation, continuous across cells, gives the same
// value to rounding; the stage kernels keep locate's exact arithmetic.
__device__ __forceinline__ bool locate_fast(const mk_snapshot_view &s, double x, double y, double z, CellPos &c) {
    const int mb = find_block(s, x, y, z);
    if (mb < 0) return false;
    c.mb = mb;
    const double *g = s.geom + 6 * (int64_t)mb;
    const double xs[3] = {x, y, z};
#pragma unroll
    for (int a = 0; a < 3; a++) {
        const double d = __ldg(g + 3 + a);
        const double q = (xs[a] - __ldg(g + a) + d) * rcp64(d);
        const double fl = floor(q);
        c.del[a] = q - fl;
        const int i = (int)fl;
        // the face test guarantees 0 <= i <= n up to rounding; clamp keeps loads in bounds
        c.idx[a] = i < 0 ? 0 : (i > s.n ? s.n : i);
    }
    return true;
}

__device__ __forceinline__ float4 ldg4(const float *p) { return __ldg(reinterpret_cast<const float4 *>(p)); }

// trilinear interpolation of the 8 primitives (athenak.py:737-752), FP64.
// Blocks whose ghosts average finer cells are read from their binary64 copy
// (the means are not float32 values; the reference holds them in float64).
template <bool EXACT>
__device__ __forceinline__ void trilinear8_impl(const mk_snapshot_view &s, const CellPos &c, double prim[8]) {
    const int n2 = s.n + 2;
    const int64_t sj = (int64_t)n2 * 8, sk = (int64_t)n2 * n2 * 8;
    const int64_t at = ((((int64_t)c.mb * n2 + c.idx[2]) * n2 + c.idx[1]) * n2 + c.idx[0]) * 8;
    const int row = s.blocks64 ? __ldg(s.block64 + c.mb) : -1;
    double v[2][2][2][8];
    if (row >= 0) {
        const double *base = s.blocks64 + at + ((int64_t)row - c.mb) * n2 * n2 * n2 * 8;
#pragma unroll
        for (int dk = 0; dk < 2; dk++)
#pragma unroll
            for (int dj = 0; dj < 2; dj++)
#pragma unroll
                for (int di = 0; di < 2; di++)
#pragma unroll
                    for (int p = 0; p < 8; p++) v[dk][dj][di][p] = __ldg(base + dk * sk + dj * sj + di * 8 + p);
    } else {
        const float *base = s.blocks + at;
#pragma unroll
        for (int dk = 0; dk < 2; dk++)
#pragma unroll
            for (int dj = 0; dj < 2; dj++)
#pragma unroll
                for (int di = 0; di < 2; di++) {
                    const float *p = base + dk * sk + dj * sj + di * 8;
                    const float4 lo = ldg4(p), hi = ldg4(p + 4);
                    v[dk][dj][di][0] = lo.x; v[dk][dj][di][1] = lo.y; v[dk][dj][di][2] = lo.z;
                    v[dk][dj][di][3] = lo.w; v[dk][dj][di][4] = hi.x; v[dk][dj][di][5] = hi.y;
                    v[dk][dj][di][6] = hi.z; v[dk][dj][di][7] = hi.w;
                }
    }
    const double d1 = c.del[0], d2 = c.del[1], d3 = c.del[2];
    // EXACT: a + (b - a) d rounded twice (no fused multiply-add), as the
    // reference evaluates it, so the interpolated primitives are
    // bit-identical; otherwise (fused render) one fused multiply-add
    auto lerp = [](double a, double b, double d) {
        return EXACT ? __dadd_rn(a, __dmul_rn(__dsub_rn(b, a), d)) : fma(b - a, d, a);
    };
#pragma unroll
    for (int p = 0; p < 8; p++) {
        const double aaa = v[0][0][0][p], aab = v[0][0][1][p], aba = v[0][1][0][p], abb = v[0][1][1][p];
        const double baa = v[1][0][0][p], bab = v[1][0][1][p], bba = v[1][1][0][p], bbb = v[1][1][1][p];
        const double daa = lerp(aaa, aab, d1);
        const double dab = lerp(aba, abb, d1);
        const double dba = lerp(baa, bab, d1);
        const double dbb = lerp(bba, bbb, d1);
        const double da = lerp(daa, dab, d2);
        const double db = lerp(dba, dbb, d2);
        prim[p] = lerp(da, db, d3);
    }
}

__device__ __forceinline__ void trilinear8(const mk_snapshot_view &s, const CellPos &c, double prim[8]) {
    trilinear8_impl<true>(s, c, prim);
}
__device__ __forceinline__ void trilinear8_fast(const mk_snapshot_view &s, const CellPos &c, double prim[8]) {
    trilinear8_impl<false>(s, c, prim);
}

// fluid scalars at one point (athenak.py:759-794); k = photon wavevector
struct FluidScalars {
    double dens, u, pitch, kdotu, b;
};

struct FluidFrame {
    double dens, u, cos_pitch, kdotu, b;
};

// the frame from metric data at the point; cos_pitch is the clamped cosine
// (the pitch angle is acos of it)
__device__ __forceinline__ FluidFrame fluid_frame_m(const double prim[8], const KerrPoint<double> &m,
                                                    const double k[4], double cos_fallback) {
    const double f = m.f, l1 = m.l1, l2 = m.l2, l3 = m.l3;
    // g^{00} = -1 - f, g^{0i} = f l_i; the lapse alpha = 1/sqrt(1 + f), the
    // Lorentz factor gamma = sqrt(G), and 1/u^0 = alpha/gamma from the two
    // reciprocal square roots (no division on the FP64 pipe)
    const double opf = 1.0 + f;
    const double alpha = rsqrt64(opf);
    const double U1 = prim[1], U2 = prim[2], U3 = prim[3];
    const double lU = l1 * U1 + l2 * U2 + l3 * U3;
    const double G = 1.0 + ((U1 * U1 + U2 * U2 + U3 * U3) + f * lU * lU);
    const double rG = rsqrt64(G);
    const double gamma = G * rG;
    const double ga_f = gamma * alpha * f;
    const double uc0 = gamma * (opf * alpha);
    const double uc1 = U1 - ga_f * l1, uc2 = U2 - ga_f * l2, uc3 = U3 - ga_f * l3;
    const double lu = uc0 + l1 * uc1 + l2 * uc2 + l3 * uc3;
    const double flu = f * lu;
    const double ud0 = -uc0 + flu, ud1 = uc1 + l1 * flu, ud2 = uc2 + l2 * flu, ud3 = uc3 + l3 * flu;
    const double B1 = prim[5], B2 = prim[6], B3 = prim[7];
    const double bc0 = B1 * ud1 + B2 * ud2 + B3 * ud3;
    const double iuc0 = alpha * rG;
    const double bc1 = (B1 + uc1 * bc0) * iuc0, bc2 = (B2 + uc2 * bc0) * iuc0, bc3 = (B3 + uc3 * bc0) * iuc0;
    const double lb = bc0 + l1 * bc1 + l2 * bc2 + l3 * bc3;
    const double flb = f * lb;
    const double bd0 = -bc0 + flb, bd1 = bc1 + l1 * flb, bd2 = bc2 + l2 * flb, bd3 = bc3 + l3 * flb;
    FluidFrame o;
    o.kdotu = k[0] * ud0 + k[1] * ud1 + k[2] * ud2 + k[3] * ud3;
    const double kdotb = k[0] * bd0 + k[1] * bd1 + k[2] * bd2 + k[3] * bd3;
    const double bdotb = bc0 * bd0 + bc1 * bd1 + bc2 * bd2 + bc3 * bd3;
    o.b = sqrt64(bdotb);
    double pitch = kdotb * rcp64(fabs(o.kdotu) * o.b);
    if (isnan(pitch)) pitch = cos_fallback;
    if (fabs(pitch) > 1.0) pitch = isinf(pitch) ? nan("") : copysign(1.0, pitch);  // x/|x|, inf/inf = NaN
    o.cos_pitch = pitch;
    o.dens = prim[0];
    o.u = prim[4];
    return o;
}

__device__ __forceinline__ FluidScalars fluid_frame(const double prim[8], double x, double y, double z,
                                                    const double k[4], double a, double cos_fallback) {
    const FluidFrame fr = fluid_frame_m(prim, kerr_point(x, y, z, a), k, cos_fallback);
    FluidScalars o;
    o.dens = fr.dens;
    o.u = fr.u;
    o.pitch = acos(fr.cos_pitch);
    o.kdotu = fr.kdotu;
    o.b = fr.b;
    return o;
}

// rlow_rhigh_model (electrons.py:32-50)
// the same with reciprocals in place of the three divisions (the fused
// FP64 render: within a few ulp of rlow_rhigh, which the stage kernel
// keeps bit-exact to the reference)
__device__ __forceinline__ double rlow_rhigh_fast(double dens, double u, double beta, double r_low,
                                                  double r_high, double gem1, double gim1) {
    const double b2 = beta * beta;
    const double T_ratio = (r_high * b2 + r_low) * rcp64(1.0 + b2);
    const double t = CL2 * (((MP * u) * gem1) * gim1);
    return t * rcp64(dens * (gim1 + gem1 * T_ratio)) * (1.0 / ME_CL_CL);
}

__device__ __forceinline__ double rlow_rhigh(double dens, double u, double beta, double r_low,
                                             double r_high, double gem1, double gim1) {
    const double b2 = beta * beta;
    const double T_ratio = (r_high * b2 + r_low) / (1.0 + b2);
    double t = CL2 * (((MP * u) * gem1) * gim1);
    t /= dens * (gim1 + gem1 * T_ratio);
    return t / ME_CL_CL;
}

// synchrotron_coefficients (transfer.py:30-86), FP64.  Frequency-independent
// parts are split out so a multi-frequency pass evaluates them once.
// per-sample factors of the synchrotron fit shared by every frequency:
// nus, Theta_e, Ne, and the reciprocals 1/nus, 1/(2 Theta_e^2), 1/Theta_e
// (quotients become products on the FP64 pipe; each within 2 ulp)
struct SynchroPre {
    double nus, th, Ne, inus, i2th2, ith;
};

__device__ __forceinline__ SynchroPre synchro_pre_sin(double Ne, double Th, double B, double sin_pitch) {
    SynchroPre p;
    const double nuc = B * (EE / TWO_PI_ME_CL);
    const double th2 = Th * Th;
    p.nus = ((TWO_NINTHS * nuc) * th2) * sin_pitch;
    p.th = Th;
    p.Ne = Ne;
    p.inus = rcp64(p.nus);
    p.i2th2 = rcp64(2.0 * th2);
    p.ith = rcp64(Th);
    return p;
}

__device__ __forceinline__ SynchroPre synchro_pre(double Ne, double Th, double B, double pitch) {
    return synchro_pre_sin(Ne, Th, B, sin(pitch));
}

// sin(acos(c)) without the two transcendentals; (1-c)(1+c) keeps full
// relative accuracy as |c| -> 1
__device__ __forceinline__ double sin_from_cos(double c) { return sqrt((1.0 - c) * (1.0 + c)); }

__device__ __forceinline__ void synchro_eval(const SynchroPre &p, double nu, bool invariant, double rescale_nu,
                                             double &em_out, double &ab_out) {
    const double X = nu * p.inus;
    // X^(1/3) and X^(1/6) = sqrt(X^(1/3)): cbrt is exact to an ulp and far
    // cheaper than pow on the FP64 pipe
    const double x3 = cbrt(X);
    const double var = exp(-x3);
    const double term = sqrt64(X) + C2_11_12 * sqrt64(x3);
    double em = p.Ne * p.nus * (term * term) * p.i2th2;
    em = em * var * (SQRT2 * PI * EE2 / THREE_CL);
    if (X > 1.e12) em = 0.0;
    if (p.th < 0.3) em = 0.0;
    const double bx = (HPL / ME_CL_CL) * nu * p.ith;
    const double Bden = (bx < 2.e-3) ? bx * (1.0 / 24.) * (24. + bx * (12. + bx * (4. + bx))) : (exp(bx) - 1.0);
    // alpha = em / B_nu with B_nu = 2 HPL nu^3 / Bden / CL^2
    const double inu = rcp64(nu);
    double ab = em * Bden * (CL2 / TWO_HPL) * (inu * inu * inu);
    if (invariant) {
        const double rn = nu * rescale_nu;
        const double irn = rcp64(rn);
        em = em * (irn * irn);
        ab = ab * rn;
    }
    em_out = isnan(em) ? 0.0 : em;
    ab_out = isnan(ab) ? 0.0 : ab;
}

}  // namespace mk

// ------------------------------------------------------------------------
// FP32 sampling and emission for the mixed-precision render.  Same
// mathematics as above, evaluated in float with the cgs prefactors folded
// into per-frequency constants so no intermediate leaves the float range
// (2 HPL / c^2 = 1.5e-47 would underflow on its own).
// ------------------------------------------------------------------------
namespace mk {

// per-frequency constants of the FP32 synchrotron (computed in FP64 once
// per ray, see synchro_consts)
struct SynchroF32 {
    float k_em;   // sqrt2 pi EE^2/(3 CL) * nu_obs: emissivity prefactor in rescaled units
    float k_bx;   // HPL nu_obs / (ME CL^2): bx = k_bx nu' / Theta_e
    float k_bnu;  // 2 HPL nu_obs^3 / CL^2: B_nu = k_bnu nu'^3 / Bden
    float inv_nu; // 1 / nu_obs (only for nus' = nus / nu_obs)
};

__device__ __forceinline__ SynchroF32 synchro_consts(double nu_obs) {
    SynchroF32 c;
    c.k_em = (float)(SQRT2 * PI * EE2 / THREE_CL * nu_obs);
    c.k_bx = (float)(HPL * nu_obs / ME_CL_CL);
    c.k_bnu = (float)(TWO_HPL * nu_obs * nu_obs * nu_obs / CL2);
    c.inv_nu = (float)(1.0 / nu_obs);
    return c;
}

// block lookup + ghost-shifted cell position in float (uniform single-level
// grid: block = floor((x - lo)/width); cells from the block's first centre)
struct CellPosF {
    int mb;
    int idx[3];
    float del[3];
};

// r_out: a Kerr-Schild radius beyond which no point of the snapshot's block
// grid lies (r <= |x| in these coordinates, so the largest corner distance
// of the grid, rounded up by 1 M, bounds it)
struct SnapF32 {
    float lo[3], inv_w[3], r_out;
};

__device__ __forceinline__ SnapF32 snap_f32(const mk_snapshot_view &s) {
    SnapF32 f;
    double rr = 0.0;
#pragma unroll
    for (int a = 0; a < 3; a++) {
        f.lo[a] = (float)s.lo[a];
        f.inv_w[a] = (float)(1.0 / s.width[a]);
        const double e = fmax(fabs(s.lo[a]), fabs(s.lo[a] + s.nb[a] * s.width[a]));
        rr += e * e;
    }
    f.r_out = (float)(sqrt(rr) + 1.0);
    return f;
}

// index of the lookup-table cell holding (x, y, z), or -1 outside the grid
__device__ __forceinline__ int64_t table_cell_f32(const mk_snapshot_view &s, const SnapF32 &sf, const float xs[3]) {
    int b[3];
#pragma unroll
    for (int a = 0; a < 3; a++) {
        const float u = (xs[a] - sf.lo[a]) * sf.inv_w[a];
        if (!(u >= 0.0f && u < (float)s.nb[a])) return -1;
        b[a] = min((int)u, s.nb[a] - 1);
    }
    return ((int64_t)b[2] * s.nb[1] + b[1]) * s.nb[0] + b[0];
}

// cell and offsets of (x, y, z) in a block with first cell centre `left`
// and reciprocal cell widths inv_dx
__device__ __forceinline__ void cell_in_block_f32(const mk_snapshot_view &s, const float xs[3], const float left[3],
                                                  const float inv_dx[3], CellPosF &c) {
#pragma unroll
    for (int a = 0; a < 3; a++) {
        const float t = (xs[a] - left[a]) * inv_dx[a] + 1.0f;  // ghost-shifted
        const float fl = floorf(t);
        int i = (int)fl;
        float d = t - fl;
        if (i < 0) { i = 0; d = 0.0f; }
        if (i > s.n) { i = s.n; d = 1.0f; }
        c.idx[a] = i;
        c.del[a] = d;
    }
}

__device__ __forceinline__ bool locate_f32(const mk_snapshot_view &s, const SnapF32 &sf, float x, float y, float z,
                                           CellPosF &c) {
    const float xs[3] = {x, y, z};
    const int64_t cell = table_cell_f32(s, sf, xs);
    if (cell < 0) return false;
    const int mb = __ldg(s.table + cell);
    if (mb < 0) return false;
    c.mb = mb;
    const float4 g0 = __ldg(reinterpret_cast<const float4 *>(s.geom_f32) + 2 * (int64_t)mb);
    const float4 g1 = __ldg(reinterpret_cast<const float4 *>(s.geom_f32) + 2 * (int64_t)mb + 1);
    const float left[3] = {g0.x, g0.y, g0.z}, inv_dx[3] = {g0.w, g1.x, g1.y};
    cell_in_block_f32(s, xs, left, inv_dx, c);
    return true;
}

// The lookup-table cell, block and block geometry of a ray's last lookup,
// kept in registers.  Consecutive steps of one ray mostly stay in one
// table cell, and then locate_f32_cached finds the cell with no memory
// access; locate_f32's two dependent loads (table, then geometry) sat on
// the near-hole phase's serial chain at every step.  Reset it (key = -1)
// whenever the ray or its snapshot changes.
struct BlockCacheF {
    int64_t key;
    int mb;
    float left[3], inv_dx[3];
};

__device__ __forceinline__ bool locate_f32_cached(const mk_snapshot_view &s, const SnapF32 &sf, float x, float y,
                                                  float z, CellPosF &c, BlockCacheF &bc) {
    const float xs[3] = {x, y, z};
    const int64_t cell = table_cell_f32(s, sf, xs);
    if (cell < 0) return false;
    if (cell != bc.key) {
        bc.key = cell;
        bc.mb = __ldg(s.table + cell);
        if (bc.mb >= 0) {
            const float4 g0 = __ldg(reinterpret_cast<const float4 *>(s.geom_f32) + 2 * (int64_t)bc.mb);
            const float4 g1 = __ldg(reinterpret_cast<const float4 *>(s.geom_f32) + 2 * (int64_t)bc.mb + 1);
            bc.left[0] = g0.x;
            bc.left[1] = g0.y;
            bc.left[2] = g0.z;
            bc.inv_dx[0] = g0.w;
            bc.inv_dx[1] = g1.x;
            bc.inv_dx[2] = g1.y;
        }
    }
    if (bc.mb < 0) return false;
    c.mb = bc.mb;
    cell_in_block_f32(s, xs, bc.left, bc.inv_dx, c);
    return true;
}

// Starts moving the 8 cells trilinear8_f32 will read for c into L1
// (prefetch.global.L1 does not stall the issuing warp), so that the sample
// taken after the next acceleration finds them there: the phases that run
// one warp per sub-partition are latency-bound, not bandwidth-bound.  c comes
// from a successful locate_f32, so every address lies in the block array.
__device__ __forceinline__ void prefetch_cells_f32(const mk_snapshot_view &s, const CellPosF &c) {
    const int n2 = s.n + 2;
    const int64_t sj = (int64_t)n2 * 8, sk = (int64_t)n2 * n2 * 8;
    const float *base = s.blocks + ((((int64_t)c.mb * n2 + c.idx[2]) * n2 + c.idx[1]) * n2 + c.idx[0]) * 8;
#pragma unroll
    for (int dk = 0; dk < 2; dk++)
#pragma unroll
        for (int dj = 0; dj < 2; dj++) {
            const float *p = base + dk * sk + dj * sj;
            asm volatile("prefetch.global.L1 [%0];" ::"l"(p));
            asm volatile("prefetch.global.L1 [%0];" ::"l"(p + 8));
        }
}

__device__ __forceinline__ void trilinear8_f32(const mk_snapshot_view &s, const CellPosF &c, float prim[8]) {
    const int n2 = s.n + 2;
    const int64_t sj = (int64_t)n2 * 8, sk = (int64_t)n2 * n2 * 8;
    const float *base = s.blocks + ((((int64_t)c.mb * n2 + c.idx[2]) * n2 + c.idx[1]) * n2 + c.idx[0]) * 8;
    // primitives in pairs (0-1, 2-3, 4-5, 6-7), lerped on paired FP32
    // instructions: each lane is fma(b - a, d, a) as in the scalar form
    float2 v[2][2][2][4];
#pragma unroll
    for (int dk = 0; dk < 2; dk++)
#pragma unroll
        for (int dj = 0; dj < 2; dj++)
#pragma unroll
            for (int di = 0; di < 2; di++) {
                const float *p = base + dk * sk + dj * sj + di * 8;
                const float4 lo = ldg4(p), hi = ldg4(p + 4);
                v[dk][dj][di][0] = make_float2(lo.x, lo.y);
                v[dk][dj][di][1] = make_float2(lo.z, lo.w);
                v[dk][dj][di][2] = make_float2(hi.x, hi.y);
                v[dk][dj][di][3] = make_float2(hi.z, hi.w);
            }
    const float2 d1 = make_float2(c.del[0], c.del[0]), d2 = make_float2(c.del[1], c.del[1]),
                 d3 = make_float2(c.del[2], c.del[2]), m1 = make_float2(-1.0f, -1.0f);
    auto lerp = [&](float2 a, float2 b, float2 d) { return __ffma2_rn(__ffma2_rn(a, m1, b), d, a); };
#pragma unroll
    for (int p = 0; p < 4; p++) {
        const float2 daa = lerp(v[0][0][0][p], v[0][0][1][p], d1);
        const float2 dab = lerp(v[0][1][0][p], v[0][1][1][p], d1);
        const float2 dba = lerp(v[1][0][0][p], v[1][0][1][p], d1);
        const float2 dbb = lerp(v[1][1][0][p], v[1][1][1][p], d1);
        const float2 da = lerp(daa, dab, d2);
        const float2 db = lerp(dba, dbb, d2);
        const float2 r = lerp(da, db, d3);
        prim[2 * p] = r.x;
        prim[2 * p + 1] = r.y;
    }
}

struct FluidF32 {
    float dens, u, cos_pitch, kdotu, b;
};

// fluid frame in float; returns the clamped cosine of the pitch angle (the
// emission needs sin(pitch) = sqrt(1 - cos^2), not the angle)
// Approximate float square root and cube root for the mixed-form emission:
// one MUFU.SQRT, and 2^(log2(x)/3) by MUFU.LG2/MUFU.EX2 (relative error
// ~1e-7 and ~1e-6; sqrt(0) = 0, cbrt(0) = 0, NaN and inf propagate).
__device__ __forceinline__ float sqrt_approx(float x) {
    float r;
    asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
__device__ __forceinline__ float cbrt_approx(float x) {
    float l, r;
    asm("lg2.approx.ftz.f32 %0, %1;" : "=f"(l) : "f"(x));
    l *= 0.333333343f;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(l));
    return r;
}

__device__ __forceinline__ FluidF32 fluid_frame_f32(const float prim[8], const KerrPoint<float> &m, const float k[4],
                                                    float cos_fallback) {
    const float f = m.f, l1 = m.l1, l2 = m.l2, l3 = m.l3;
    const float alpha = rsqrt_ftz(1.0f + f);
    const float U1 = prim[1], U2 = prim[2], U3 = prim[3];
    const float lU = l1 * U1 + l2 * U2 + l3 * U3;
    const float gamma = sqrt_approx(1.0f + ((U1 * U1 + U2 * U2 + U3 * U3) + f * lU * lU));
    const float ga_f = gamma * alpha * f;
    const float uc0 = gamma * ((1.0f + f) * alpha);  // gamma / alpha with alpha = 1/sqrt(1 + f)
    const float uc1 = U1 - ga_f * l1, uc2 = U2 - ga_f * l2, uc3 = U3 - ga_f * l3;
    const float lu = uc0 + l1 * uc1 + l2 * uc2 + l3 * uc3;
    const float flu = f * lu;
    const float ud0 = -uc0 + flu, ud1 = uc1 + l1 * flu, ud2 = uc2 + l2 * flu, ud3 = uc3 + l3 * flu;
    const float B1 = prim[5], B2 = prim[6], B3 = prim[7];
    const float bc0 = B1 * ud1 + B2 * ud2 + B3 * ud3;
    const float iuc0 = rcp_ftz(uc0);
    const float bc1 = (B1 + uc1 * bc0) * iuc0, bc2 = (B2 + uc2 * bc0) * iuc0, bc3 = (B3 + uc3 * bc0) * iuc0;
    const float lb = bc0 + l1 * bc1 + l2 * bc2 + l3 * bc3;
    const float flb = f * lb;
    const float bd0 = -bc0 + flb, bd1 = bc1 + l1 * flb, bd2 = bc2 + l2 * flb, bd3 = bc3 + l3 * flb;
    FluidF32 o;
    o.kdotu = k[0] * ud0 + k[1] * ud1 + k[2] * ud2 + k[3] * ud3;
    const float kdotb = k[0] * bd0 + k[1] * bd1 + k[2] * bd2 + k[3] * bd3;
    const float bdotb = bc0 * bd0 + bc1 * bd1 + bc2 * bd2 + bc3 * bd3;
    const float bmag = sqrt_approx(bdotb);
    float cp = fdiv(kdotb, fabsf(o.kdotu) * bmag);
    if (isnan(cp)) cp = cos_fallback;
    o.cos_pitch = fminf(fmaxf(cp, -1.0f), 1.0f);
    o.dens = prim[0];
    o.u = prim[4];
    o.b = bmag;
    return o;
}

}  // namespace mk
