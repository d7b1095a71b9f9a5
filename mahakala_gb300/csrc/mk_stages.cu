// mk_stages.cu -- per-stage kernels behind the reference's step-by-step API
// (get_fluid_scalars_from_geodesics, rlow_rhigh_model,
// synchrotron_coefficients, solve_specific_intensity, ...) and the snapshot
// builder.  The fused render does not use these; they keep the reference's
// stage-by-stage call sequence available on the device.
#include "mk_common.cuh"
#include "mk_fluid.cuh"

namespace mk {

// Block of a mesh at (level, i, j, k) by binary search of the sorted keys,
// -1 if there is none (negative or out-of-range locations included).
__device__ __forceinline__ int mesh_find(const int64_t *__restrict__ keys, const int32_t *__restrict__ key_block,
                                         int nmb, int lv, int i, int j, int k) {
    const int lim = 1 << 18;
    if (lv < 0 || lv >= 512 || i < 0 || j < 0 || k < 0 || i >= lim || j >= lim || k >= lim) return -1;
    const int64_t want = MK_MESH_KEY(lv, i, j, k);
    int lo = 0, hi = nmb - 1;
    while (lo <= hi) {
        const int mid = (lo + hi) >> 1;
        const int64_t v = keys[mid];
        if (v == want) return key_block[mid];
        if (v < want) lo = mid + 1;
        else hi = mid - 1;
    }
    return -1;
}

__device__ __forceinline__ int py_floordiv2(int x) { return x >= 0 ? x / 2 : -((1 - x) / 2); }

// One ghost-filled meshblock cell: one thread per padded cell (mb, k, j, i).
// The ghost rules of load_athenak_meshblocks (grmhd/athenak.py:108-158,
// 208-525), in order: same-level neighbour (copy of its adjacent cells);
// coarser neighbour (each coarse cell copied to the 2 fine ghosts it covers
// per transverse axis, the half chosen by the parity of t + d); finer
// neighbours (mean of 2x2x2 fine cells: eight terms value/8 in float32,
// summed in binary64, i over j over k, where an edge region's transverse
// source is one cell for the first term and then the every-other-cell
// offset of the previous term, as the reference's loop reads it); zero.
__global__ void snapshot_build_kernel(mk_mesh_desc m, float *__restrict__ out) {
    const int n = m.n, n2 = n + 2, h = n / 2;
    const int64_t total = (int64_t)m.nmb * n2 * n2 * n2;
    const int64_t cell = (int64_t)n * n * n;
    const int64_t pstride = (int64_t)m.nmb * cell;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
         e += (int64_t)gridDim.x * blockDim.x) {
        int64_t q = e;
        int c[3];
        c[0] = (int)(q % n2); q /= n2;
        c[1] = (int)(q % n2); q /= n2;
        c[2] = (int)(q % n2); q /= n2;
        const int mb = (int)q;
        int d[3];
#pragma unroll
        for (int a = 0; a < 3; a++) d[a] = c[a] == 0 ? -1 : (c[a] == n + 1 ? 1 : 0);
        double v[8];
        auto load = [&](int blk, const int src[3], int p) -> float {
            const int64_t off = (int64_t)blk * cell + ((int64_t)src[2] * n + src[1]) * n + src[0];
            return p < 5 ? m.uov[(int64_t)p * pstride + off] : m.B[(int64_t)(p - 5) * pstride + off];
        };
        if (!(d[0] || d[1] || d[2])) {
            const int src[3] = {c[0] - 1, c[1] - 1, c[2] - 1};
#pragma unroll
            for (int p = 0; p < 8; p++) v[p] = (double)load(mb, src, p);
        } else {
            const int lv = m.levels[mb];
            const int t[3] = {m.locs[3 * mb], m.locs[3 * mb + 1], m.locs[3 * mb + 2]};
            int nb = mesh_find(m.keys, m.key_block, m.nmb, lv, t[0] + d[0], t[1] + d[1], t[2] + d[2]);
            if (nb >= 0) {  // same level
                int src[3];
#pragma unroll
                for (int a = 0; a < 3; a++) src[a] = d[a] == 1 ? 0 : (d[a] == -1 ? n - 1 : c[a] - 1);
#pragma unroll
                for (int p = 0; p < 8; p++) v[p] = (double)load(nb, src, p);
            } else if ((nb = mesh_find(m.keys, m.key_block, m.nmb, lv - 1, py_floordiv2(t[0] + d[0]),
                                       py_floordiv2(t[1] + d[1]), py_floordiv2(t[2] + d[2]))) >= 0) {
                int src[3];  // coarser neighbour
#pragma unroll
                for (int a = 0; a < 3; a++) {
                    const int odd = (t[a] + d[a]) & 1;  // == Python's % 2 for either sign
                    src[a] = d[a] == 1 ? (odd ? h : 0) : (d[a] == -1 ? (odd ? n - 1 : h - 1) : (odd ? h : 0) + (c[a] - 1) / 2);
                }
#pragma unroll
                for (int p = 0; p < 8; p++) v[p] = (double)load(nb, src, p);
            } else if (mesh_find(m.keys, m.key_block, m.nmb, lv + 1, 2 * (t[0] + d[0]), 2 * (t[1] + d[1]),
                                 2 * (t[2] + d[2])) >= 0) {
                // finer neighbours: the fine block holding this ghost cell's 2x2x2 cells
                int blk[3], s0[3], mz[3], nz = 0;
#pragma unroll
                for (int a = 0; a < 3; a++) {
                    nz += d[a] != 0;
                    const int ep = d[a] == 0 ? (c[a] - 1) / h : 0;
                    blk[a] = 2 * (t[a] + d[a]) + (d[a] == -1 ? 1 : 0) + ep;
                    s0[a] = d[a] == -1 ? n - 2 : 0;
                    mz[a] = d[a] == 0 ? (c[a] - 1) - ep * h : 0;
                }
                nb = mesh_find(m.keys, m.key_block, m.nmb, lv + 1, blk[0], blk[1], blk[2]);
#pragma unroll
                for (int p = 0; p < 8; p++) v[p] = 0.0;
                if (nb >= 0) {
                    int prev[3] = {0, 0, 0};
                    for (int step = 0; step < 8; step++) {
                        const int w[3] = {(step >> 2) & 1, (step >> 1) & 1, step & 1};
                        int src[3];
#pragma unroll
                        for (int a = 0; a < 3; a++) {
                            if (d[a] != 0) src[a] = s0[a] + w[a];
                            else if (nz == 2) src[a] = step == 0 ? 0 : prev[a] + 2 * mz[a];
                            else src[a] = w[a] + 2 * mz[a];
                        }
#pragma unroll
                        for (int p = 0; p < 8; p++) v[p] += (double)(load(nb, src, p) / 8.0f);
#pragma unroll
                        for (int a = 0; a < 3; a++) prev[a] = w[a];
                    }
                }
            } else {
#pragma unroll
                for (int p = 0; p < 8; p++) v[p] = 0.0;
            }
        }
        float4 *o = reinterpret_cast<float4 *>(out + e * 8);
        o[0] = make_float4((float)v[0], (float)v[1], (float)v[2], (float)v[3]);
        o[1] = make_float4((float)v[4], (float)v[5], (float)v[6], (float)v[7]);
        if (m.blocks64 && m.block64[mb] >= 0) {
            double *o64 = m.blocks64 + ((int64_t)m.block64[mb] * n2 * n2 * n2 + (e - (int64_t)mb * n2 * n2 * n2)) * 8;
#pragma unroll
            for (int p = 0; p < 8; p++) o64[p] = v[p];
        }
    }
}

// float copy of the per-block geometry for the mixed-precision sampler:
// (x1v[0], x2v[0], x3v[0], 1/dx1, 1/dx2, 1/dx3, 0, 0) per block
__global__ void geom_f32_kernel(const double *__restrict__ geom, int nmb, float *__restrict__ out) {
    const int mb = blockIdx.x * blockDim.x + threadIdx.x;
    if (mb >= nmb) return;
    const double *g = geom + 6 * (int64_t)mb;
    float4 *o = reinterpret_cast<float4 *>(out + 8 * (int64_t)mb);
    o[0] = make_float4((float)g[0], (float)g[1], (float)g[2], (float)(1.0 / g[3]));
    o[1] = make_float4((float)(1.0 / g[4]), (float)(1.0 / g[5]), 0.0f, 0.0f);
}

__global__ void fluid_scalars_kernel(mk_snapshot_view sv, double a, const double *__restrict__ S, int64_t npts,
                                     double cos_fallback, double *__restrict__ out) {
    const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (p >= npts) return;
    const double *s = S + 8 * p;
    double prim[8];
    CellPos c;
    if (locate(sv, s[1], s[2], s[3], c)) trilinear8(sv, c, prim);
    else
#pragma unroll
        for (int q = 0; q < 8; q++) prim[q] = 0.0;
    const double k[4] = {s[4], s[5], s[6], s[7]};
    const FluidScalars fs = fluid_frame(prim, s[1], s[2], s[3], k, a, cos_fallback);
    out[5 * p + 0] = fs.dens;
    out[5 * p + 1] = fs.u;
    out[5 * p + 2] = fs.pitch;
    out[5 * p + 3] = fs.kdotu;
    out[5 * p + 4] = fs.b;
}

__global__ void fluid_prims_kernel(mk_snapshot_view sv, const double *__restrict__ S, int64_t npts,
                                   double *__restrict__ out, int32_t *__restrict__ block) {
    const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (p >= npts) return;
    const double *s = S + 8 * p;
    double prim[8];
    CellPos c;
    int mb = -1;
    if (locate(sv, s[1], s[2], s[3], c)) {
        trilinear8(sv, c, prim);
        mb = c.mb;
    } else {
#pragma unroll
        for (int q = 0; q < 8; q++) prim[q] = 0.0;
    }
#pragma unroll
    for (int q = 0; q < 8; q++) out[8 * p + q] = prim[q];
    if (block) block[p] = mb;
}

__global__ void rlow_rhigh_kernel(const double *__restrict__ dens, const double *__restrict__ u,
                                  const double *__restrict__ beta, int64_t n, double r_low, double r_high,
                                  double gem1, double gim1, double *__restrict__ out) {
    const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (p >= n) return;
    out[p] = rlow_rhigh(dens[p], u[p], beta[p], r_low, r_high, gem1, gim1);
}

__global__ void synchrotron_kernel(const double *__restrict__ Ne, const double *__restrict__ Th,
                                   const double *__restrict__ B, const double *__restrict__ pitch,
                                   const double *__restrict__ nu, int64_t n, int invariant, double rescale_nu,
                                   double *__restrict__ em, double *__restrict__ ab) {
    const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (p >= n) return;
    const SynchroPre sp = synchro_pre(Ne[p], Th[p], B[p], pitch[p]);
    double e, b;
    synchro_eval(sp, nu[p], invariant != 0, rescale_nu, e, b);
    em[p] = e;
    ab[p] = b;
}

// backward explicit Euler (transfer.py:106-119), one thread per pixel
__global__ void solve_intensity_kernel(const double *__restrict__ em, const double *__restrict__ ab,
                                       const double *__restrict__ dt, int64_t nsteps, int64_t npx, double L,
                                       double *__restrict__ I, double *__restrict__ dIs) {
    const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (p >= npx) return;
    double Iv = 0.0;
    for (int64_t i = nsteps - 1, r = 0; i >= 1; i--, r++) {
        const double dI = (-dt[(i - 1) * npx + p]) * L * (em[i * npx + p] - (ab[i * npx + p] * Iv));
        Iv += dI;
        if (dIs) dIs[r * npx + p] = dI;
    }
    I[p] = Iv;
}

__global__ void attenuated_kernel(const double *__restrict__ em, const double *__restrict__ ab,
                                  const double *__restrict__ dt, int64_t nsteps, int64_t npx, double L,
                                  double *__restrict__ out) {
    const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (p >= npx) return;
    double tau = 0.0;
    for (int64_t i = 1; i < nsteps; i++) {
        const double d = dt[(i - 1) * npx + p];
        const double src = -em[i * npx + p] * d * L;
        const double dtau = ab[i * npx + p] * d * L;
        out[(i - 1) * npx + p] = exp(-tau) * src;
        tau = tau - dtau;
    }
}

}  // namespace mk

using namespace mk;

static size_t blocks_bytes(int32_t nmb, int32_t n) {
    const size_t n2 = (size_t)n + 2;
    return (size_t)nmb * n2 * n2 * n2 * 8 * sizeof(float);
}

extern "C" size_t mk_snapshot_bytes(int32_t nmb, int32_t n) {
    if (nmb <= 0 || n <= 0) return 0;
    return blocks_bytes(nmb, n) + (size_t)nmb * 8 * sizeof(float);
}

extern "C" int mk_snapshot_build(const mk_mesh_desc *mesh, void *storage_dev, size_t storage_bytes,
                                 mk_snapshot_view *view_out, void *stream) {
    MK_REQUIRE(mesh && storage_dev && view_out, MK_ERR_ARG, "mk_snapshot_build: null pointer");
    const mk_mesh_desc &m = *mesh;
    MK_REQUIRE(m.uov && m.B && m.locs && m.levels && m.keys && m.key_block && m.geom && m.faces && m.table,
               MK_ERR_ARG, "mk_snapshot_build: null mesh array");
    MK_REQUIRE(m.nmb > 0 && m.n >= 2 && m.n % 2 == 0, MK_ERR_ARG,
               "mk_snapshot_build: need nmb > 0 and an even n >= 2 (n = %d)", (int)m.n);
    MK_REQUIRE(m.nb[0] > 0 && m.nb[1] > 0 && m.nb[2] > 0 && (int64_t)m.nb[0] * m.nb[1] * m.nb[2] >= m.nmb,
               MK_ERR_ARG, "mk_snapshot_build: block table too small");
    MK_REQUIRE((m.n64 > 0) == (m.blocks64 != nullptr) && (m.blocks64 == nullptr) == (m.block64 == nullptr),
               MK_ERR_ARG, "mk_snapshot_build: blocks64, block64 and n64 go together");
    MK_REQUIRE(storage_bytes >= mk_snapshot_bytes(m.nmb, m.n), MK_ERR_ARG,
               "mk_snapshot_build: storage of %zu bytes, need %zu", storage_bytes, mk_snapshot_bytes(m.nmb, m.n));
    MK_REQUIRE(((uintptr_t)storage_dev & 15) == 0, MK_ERR_ARG, "mk_snapshot_build: storage not 16-byte aligned");
    const int64_t total = (int64_t)m.nmb * (m.n + 2) * (m.n + 2) * (m.n + 2);
    int64_t grid = (total + 255) / 256;
    const int64_t cap = (int64_t)device_sm_count() * 16;
    if (grid > cap) grid = cap;
    snapshot_build_kernel<<<(unsigned)grid, 256, 0, as_stream(stream)>>>(m, (float *)storage_dev);
    MK_LAUNCHED("snapshot_build_kernel");
    float *gf = (float *)((char *)storage_dev + blocks_bytes(m.nmb, m.n));
    geom_f32_kernel<<<grid_for(m.nmb, 128), 128, 0, as_stream(stream)>>>(m.geom, m.nmb, gf);
    MK_LAUNCHED("geom_f32_kernel");
    mk_snapshot_view v;
    v.blocks = (const float *)storage_dev;
    v.geom = m.geom;
    v.geom_f32 = gf;
    v.faces = m.faces;
    v.table = m.table;
    v.blocks64 = m.blocks64;
    v.block64 = m.block64;
    v.nmb = m.nmb;
    v.n = m.n;
    v.pad0 = 0;
    for (int a = 0; a < 3; a++) {
        v.nb[a] = m.nb[a];
        v.lo[a] = m.lo[a];
        v.width[a] = m.width[a];
    }
    *view_out = v;
    return MK_OK;
}

extern "C" int mk_fluid_scalars(const mk_snapshot_view *view, double bhspin, const double *S_dev, int64_t npts,
                                double cos_fallback, double *out_dev, void *stream) {
    MK_REQUIRE(view && S_dev && out_dev, MK_ERR_ARG, "mk_fluid_scalars: null pointer");
    MK_REQUIRE(npts >= 0, MK_ERR_ARG, "mk_fluid_scalars: negative size");
    if (npts == 0) return MK_OK;
    fluid_scalars_kernel<<<grid_for(npts, 128), 128, 0, as_stream(stream)>>>(*view, bhspin, S_dev, npts,
                                                                           cos_fallback, out_dev);
    MK_LAUNCHED("fluid_scalars_kernel");
    return MK_OK;
}

extern "C" int mk_fluid_prims(const mk_snapshot_view *view, const double *S_dev, int64_t npts, double *out_dev,
                              int32_t *block_dev, void *stream) {
    MK_REQUIRE(view && S_dev && out_dev, MK_ERR_ARG, "mk_fluid_prims: null pointer");
    MK_REQUIRE(npts >= 0, MK_ERR_ARG, "mk_fluid_prims: negative size");
    if (npts == 0) return MK_OK;
    fluid_prims_kernel<<<grid_for(npts, 128), 128, 0, as_stream(stream)>>>(*view, S_dev, npts, out_dev, block_dev);
    MK_LAUNCHED("fluid_prims_kernel");
    return MK_OK;
}

extern "C" int mk_rlow_rhigh(const double *dens_dev, const double *u_dev, const double *beta_dev, int64_t n,
                             double r_low, double r_high, double electron_gamma_m1, double ion_gamma_m1,
                             double *theta_dev, void *stream) {
    MK_REQUIRE(dens_dev && u_dev && beta_dev && theta_dev, MK_ERR_ARG, "mk_rlow_rhigh: null pointer");
    MK_REQUIRE(n >= 0, MK_ERR_ARG, "mk_rlow_rhigh: negative size");
    if (n == 0) return MK_OK;
    rlow_rhigh_kernel<<<grid_for(n, 256), 256, 0, as_stream(stream)>>>(dens_dev, u_dev, beta_dev, n, r_low, r_high,
                                                                     electron_gamma_m1, ion_gamma_m1, theta_dev);
    MK_LAUNCHED("rlow_rhigh_kernel");
    return MK_OK;
}

extern "C" int mk_synchrotron(const double *Ne_dev, const double *theta_dev, const double *B_dev,
                              const double *pitch_dev, const double *nu_dev, int64_t n, int32_t invariant,
                              double rescale_nu, double *em_dev, double *ab_dev, void *stream) {
    MK_REQUIRE(Ne_dev && theta_dev && B_dev && pitch_dev && nu_dev && em_dev && ab_dev, MK_ERR_ARG,
               "mk_synchrotron: null pointer");
    MK_REQUIRE(n >= 0, MK_ERR_ARG, "mk_synchrotron: negative size");
    if (n == 0) return MK_OK;
    synchrotron_kernel<<<grid_for(n, 128), 128, 0, as_stream(stream)>>>(Ne_dev, theta_dev, B_dev, pitch_dev, nu_dev,
                                                                      n, invariant, rescale_nu, em_dev, ab_dev);
    MK_LAUNCHED("synchrotron_kernel");
    return MK_OK;
}

extern "C" int mk_solve_intensity(const double *em_dev, const double *ab_dev, const double *dt_dev, int64_t nsteps,
                                  int64_t npx, double L_unit, double *I_dev, double *dIs_dev, void *stream) {
    MK_REQUIRE(em_dev && ab_dev && dt_dev && I_dev, MK_ERR_ARG, "mk_solve_intensity: null pointer");
    MK_REQUIRE(nsteps >= 0 && npx >= 0, MK_ERR_ARG, "mk_solve_intensity: negative size");
    if (npx == 0) return MK_OK;
    solve_intensity_kernel<<<grid_for(npx, 128), 128, 0, as_stream(stream)>>>(em_dev, ab_dev, dt_dev, nsteps, npx,
                                                                            L_unit, I_dev, dIs_dev);
    MK_LAUNCHED("solve_intensity_kernel");
    return MK_OK;
}

extern "C" int mk_attenuated_emissivity(const double *em_dev, const double *ab_dev, const double *dt_dev,
                                        int64_t nsteps, int64_t npx, double L_unit, double *out_dev, void *stream) {
    MK_REQUIRE(em_dev && ab_dev && dt_dev && out_dev, MK_ERR_ARG, "mk_attenuated_emissivity: null pointer");
    MK_REQUIRE(nsteps >= 0 && npx >= 0, MK_ERR_ARG, "mk_attenuated_emissivity: negative size");
    if (npx == 0 || nsteps < 2) return MK_OK;
    attenuated_kernel<<<grid_for(npx, 128), 128, 0, as_stream(stream)>>>(em_dev, ab_dev, dt_dev, nsteps, npx, L_unit,
                                                                       out_dev);
    MK_LAUNCHED("attenuated_kernel");
    return MK_OK;
}
