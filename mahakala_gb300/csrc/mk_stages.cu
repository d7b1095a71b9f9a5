// mk_stages.cu -- per-stage kernels behind the reference's step-by-step API
// (get_fluid_scalars_from_geodesics, rlow_rhigh_model,
// synchrotron_coefficients, solve_specific_intensity, ...) and the snapshot
// builder.  The fused render does not use these; they keep the reference's
// stage-by-stage call sequence available on the device.
#include "mk_common.cuh"
#include "mk_fluid.cuh"

namespace mk {

// ghost-filled AoS meshblocks from AthenaK arrays: one thread per padded
// cell (mb, k, j, i); same-level neighbour copy, zeros at the domain edge
// (grmhd/athenak.py:108-127, 217-233)
__global__ void snapshot_build_kernel(const float *__restrict__ uov, const float *__restrict__ B,
                                      const int32_t *__restrict__ locs, const int32_t *__restrict__ table, int nmb,
                                      int n, int nb0, int nb1, int nb2, float *__restrict__ out) {
    const int n2 = n + 2;
    const int64_t total = (int64_t)nmb * n2 * n2 * n2;
    const int64_t cell = (int64_t)n * n * n;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
         e += (int64_t)gridDim.x * blockDim.x) {
        int64_t t = e;
        const int i = (int)(t % n2); t /= n2;
        const int j = (int)(t % n2); t /= n2;
        const int k = (int)(t % n2); t /= n2;
        const int mb = (int)t;
        const int di = i == 0 ? -1 : (i == n + 1 ? 1 : 0);
        const int dj = j == 0 ? -1 : (j == n + 1 ? 1 : 0);
        const int dk = k == 0 ? -1 : (k == n + 1 ? 1 : 0);
        int src = mb;
        if (di || dj || dk) {
            const int ti = locs[3 * mb] + di, tj = locs[3 * mb + 1] + dj, tk = locs[3 * mb + 2] + dk;
            src = (ti < 0 || tj < 0 || tk < 0 || ti >= nb0 || tj >= nb1 || tk >= nb2)
                      ? -1
                      : table[((int64_t)tk * nb1 + tj) * nb0 + ti];
        }
        float v[8];
        if (src < 0) {
#pragma unroll
            for (int p = 0; p < 8; p++) v[p] = 0.0f;
        } else {
            const int si = di == 1 ? 0 : (di == -1 ? n - 1 : i - 1);
            const int sj = dj == 1 ? 0 : (dj == -1 ? n - 1 : j - 1);
            const int sk = dk == 1 ? 0 : (dk == -1 ? n - 1 : k - 1);
            const int64_t off = (int64_t)src * cell + ((int64_t)sk * n + sj) * n + si;
#pragma unroll
            for (int p = 0; p < 5; p++) v[p] = uov[(int64_t)p * nmb * cell + off];
#pragma unroll
            for (int p = 0; p < 3; p++) v[5 + p] = B[(int64_t)p * nmb * cell + off];
        }
        float4 *o = reinterpret_cast<float4 *>(out + e * 8);
        o[0] = make_float4(v[0], v[1], v[2], v[3]);
        o[1] = make_float4(v[4], v[5], v[6], v[7]);
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

extern "C" int mk_snapshot_build(const float *uov_dev, const float *B_dev, const int32_t *locs_dev,
                                 const double *geom_dev, const double *faces_dev, const int32_t *table_dev,
                                 int32_t nmb, int32_t n, const int32_t nb[3], const double lo[3],
                                 const double width[3], void *storage_dev, size_t storage_bytes,
                                 mk_snapshot_view *view_out, void *stream) {
    MK_REQUIRE(uov_dev && B_dev && locs_dev && geom_dev && faces_dev && table_dev && nb && lo && width &&
                   storage_dev && view_out,
               MK_ERR_ARG, "mk_snapshot_build: null pointer");
    MK_REQUIRE(nmb > 0 && n >= 2, MK_ERR_ARG, "mk_snapshot_build: need nmb > 0 and n >= 2");
    MK_REQUIRE(nb[0] > 0 && nb[1] > 0 && nb[2] > 0 && (int64_t)nb[0] * nb[1] * nb[2] >= nmb, MK_ERR_ARG,
               "mk_snapshot_build: block grid too small");
    MK_REQUIRE(storage_bytes >= mk_snapshot_bytes(nmb, n), MK_ERR_ARG,
               "mk_snapshot_build: storage of %zu bytes, need %zu", storage_bytes, mk_snapshot_bytes(nmb, n));
    MK_REQUIRE(((uintptr_t)storage_dev & 15) == 0, MK_ERR_ARG, "mk_snapshot_build: storage not 16-byte aligned");
    const int64_t total = (int64_t)nmb * (n + 2) * (n + 2) * (n + 2);
    int64_t grid = (total + 255) / 256;
    const int64_t cap = (int64_t)device_sm_count() * 16;
    if (grid > cap) grid = cap;
    snapshot_build_kernel<<<(unsigned)grid, 256, 0, as_stream(stream)>>>(uov_dev, B_dev, locs_dev, table_dev, nmb, n,
                                                                       nb[0], nb[1], nb[2], (float *)storage_dev);
    MK_LAUNCHED("snapshot_build_kernel");
    float *gf = (float *)((char *)storage_dev + blocks_bytes(nmb, n));
    geom_f32_kernel<<<grid_for(nmb, 128), 128, 0, as_stream(stream)>>>(geom_dev, nmb, gf);
    MK_LAUNCHED("geom_f32_kernel");
    mk_snapshot_view v;
    v.blocks = (const float *)storage_dev;
    v.geom = geom_dev;
    v.geom_f32 = gf;
    v.faces = faces_dev;
    v.table = table_dev;
    v.nmb = nmb;
    v.n = n;
    v.pad0 = 0;
    for (int a = 0; a < 3; a++) {
        v.nb[a] = nb[a];
        v.lo[a] = lo[a];
        v.width[a] = width[a];
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
