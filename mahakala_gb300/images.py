"""Image rendering: ``make_image`` (mahakala/images.py:30-144) and the
multi-request ``render_requests`` behind it.

The whole per-ray path -- camera, geodesics, GRMHD sampling, electron
temperature, synchrotron, sigma cut, transfer -- runs in one persistent
sm_103a kernel (``mk_render``); no trajectory is materialised, so
``max_chunk_bytes`` (the reference's memory knob) has nothing to bound and
is accepted for compatibility only.
"""

from dataclasses import dataclass, field

import numpy as np
import torch

from . import _lib
from ._device import device, ptr, stream_ptr
from .constants import JY, Msun
from .geodesics import make_camera, step_policy

__all__ = ["make_image", "RenderRequest", "PreparedRender", "render_requests", "image_flux_jy", "step_diagnostics"]

PRECISIONS = {"fp64": _lib.MK_FP64, "mixed": _lib.MK_MIXED, "mixed_df": _lib.MK_MIXED_DF,
              "mixed_strict": _lib.MK_MIXED_STRICT}


@dataclass
class RenderRequest:
    """Arguments of make_image for one image (one or more frequencies)."""
    model: object                      # AthenakFluidModel (resident snapshot)
    camera_inclination: float = 60
    camera_distance: float = 1000
    mass_scale: float = 1.e26
    M_bh: float = 6.2e9 * Msun
    r_high: float = 40
    observing_frequency: object = 230.e9   # scalar or a list of up to 4 frequencies
    fov: float = 20
    resolution: int = 160
    max_nsteps: int = 10000
    r_low: float = 1
    bhspin: float = None               # default: the model's spin
    div: float = 40.
    tol: float = 1e-4
    rows: int = 0                      # > 0: per-step diagnostic rows (FP64 form), see step_diagnostics
    out: dict = field(default_factory=dict)

    @property
    def freqs(self):
        return np.atleast_1d(np.asarray(self.observing_frequency, dtype=np.float64))

    @property
    def npx(self):
        return int(self.resolution) ** 2


def _fill_request(req, rq, snap_index, image, nsteps, status, offset, rows=None):
    model = req.model
    a = model.bhspin if req.bhspin is None else req.bhspin
    if model.fluid_gamma is None:
        # images.py:88 needs fluid_gamma (None raises a TypeError there)
        raise TypeError("fluid_model.fluid_gamma must be set to render an image")
    freqs = req.freqs
    if not 1 <= len(freqs) <= _lib.MK_MAX_NU:
        raise ValueError(f"1..{_lib.MK_MAX_NU} observing frequencies per request")
    rq.camera = make_camera(a, req.camera_inclination, req.camera_distance, -req.fov / 2., req.fov / 2.,
                            req.resolution)
    rq.policy = step_policy(req.max_nsteps, req.div, req.tol)
    rq.fluid_gamma = float(model.fluid_gamma)
    rq.r_low, rq.r_high = float(req.r_low), float(req.r_high)
    rq.electron_gamma_m1, rq.ion_gamma_m1 = 4. / 3 - 1., 5. / 3 - 1.
    units = model.get_units(req.M_bh, req.mass_scale)
    rq.Ne_unit, rq.B_unit, rq.L_unit = units["Ne_unit"], units["B_unit"], units["L_unit"]
    rq.cos_fallback_pitch = float(np.cos(np.pi / 3.))
    rq.sigma_cut = 100.
    rq.nnu = len(freqs)
    rq.snapshot = snap_index
    for i, f in enumerate(freqs):
        rq.nu[i] = float(f)
    rq.image, rq.nsteps, rq.status = ptr(image), ptr(nsteps), ptr(status)
    rq.ray_offset = int(offset)
    if rows is not None:
        em, ab, dt = rows
        rq.rows_em, rq.rows_ab, rq.rows_dt, rq.rows = ptr(em), ptr(ab), ptr(dt), int(dt.shape[0])


class PreparedRender:
    """A batch of requests laid out on the device once: the request table,
    the snapshot views, the output images and the launch workspace.
    ``launch()`` enqueues the single persistent render kernel; it can be
    called repeatedly (each call overwrites the outputs)."""

    def __init__(self, requests, precision="fp64", with_steps=False):
        if not requests:
            raise ValueError("no requests")
        dev = device()
        self.requests = list(requests)
        self.precision = PRECISIONS[precision]
        snaps, snap_index = [], {}
        for r in requests:
            key = id(r.model.snapshot)
            if key not in snap_index:
                snap_index[key] = len(snaps)
                snaps.append(r.model.snapshot)
        table = (_lib.Request * len(requests))()
        offset = 0
        self.images = []
        for i, r in enumerate(requests):
            img = torch.empty((len(r.freqs), r.resolution, r.resolution), dtype=torch.float64, device=dev)
            ns = st = None
            if with_steps or r.rows:
                ns = torch.empty((r.resolution, r.resolution), dtype=torch.int32, device=dev)
                st = torch.empty((r.resolution, r.resolution), dtype=torch.int32, device=dev)
            rows = None
            if r.rows:
                if precision != "fp64":
                    raise ValueError("per-step diagnostic rows come from the FP64 form only")
                nr = min(int(r.rows), int(r.max_nsteps))
                rows = (torch.zeros((len(r.freqs), nr, r.npx), dtype=torch.float64, device=dev),
                        torch.zeros((len(r.freqs), nr, r.npx), dtype=torch.float64, device=dev),
                        torch.zeros((nr, r.npx), dtype=torch.float64, device=dev))
                r.out["rows_em"], r.out["rows_ab"], r.out["rows_dt"] = rows
            _fill_request(r, table[i], snap_index[id(r.model.snapshot)], img, ns, st, offset, rows)
            if r.rows and not with_steps:
                r.out["nsteps"], r.out["status"] = ns, st
            r.out["image"] = img
            if with_steps:
                r.out["nsteps"], r.out["status"] = ns, st
            self.images.append(img)
            offset += r.npx
        self.total_rays = offset
        self.table_bytes = bytes(table)
        # the request table goes up from pinned memory (a pageable copy
        # stages through the driver); the copy completes before the
        # constructor returns, so a launch on any stream finds it
        self._table_host = torch.frombuffer(bytearray(self.table_bytes), dtype=torch.uint8).pin_memory()
        self.reqs_dev = torch.empty(len(self.table_bytes), dtype=torch.uint8, device=dev)
        self.reqs_dev.copy_(self._table_host)
        self.snaps_dev = torch.cat([sn.view_dev for sn in snaps]) if len(snaps) > 1 else snaps[0].view_dev
        self.nsnap = len(snaps)
        nbytes = _lib.load().mk_render_workspace_bytes(self.total_rays, self.precision)
        # mk_render clears the counter header itself; the queue records are
        # written before they are read
        self.ws = torch.empty((nbytes + 7) // 8, dtype=torch.int64, device=dev)

    def launch(self, stream=None):
        _lib.call("mk_render", ptr(self.reqs_dev), len(self.requests), self.total_rays, ptr(self.snaps_dev),
                  self.nsnap, self.precision, ptr(self.ws), self.ws.numel() * 8, stream_ptr(stream))
        return self.images

    def check(self):
        """Raise MKError (MK_ERR_TIMEOUT) if a bounded wait of the last
        launch's near-hole pipeline ran out, which leaves its images invalid
        (syncs).  Never expected; the limit only keeps a fault from hanging
        the GPU."""
        n = int(self.ws[_lib.MK_WS_ERROR].item())
        if n:
            raise _lib.MKError(_lib.MK_ERR_TIMEOUT,
                               f"mk_render: {n} waits of the near-hole pipeline ran out; the images are invalid")

    def work_totals(self):
        """(accepted steps, in-snapshot samples) of the last launch (syncs)."""
        w = self.ws[:32].cpu()
        return int(w[_lib.MK_WS_STEPS]), int(w[_lib.MK_WS_SAMPLES])

    def precision_split(self):
        """(rays handed to the near-hole phase, rays that left it outward,
        steps taken near the hole) of the last mixed-form launch (syncs)."""
        w = self.ws[:32].cpu()
        return int(w[_lib.MK_WS_TO_FP64]), int(w[_lib.MK_WS_TO_FP32]), int(w[_lib.MK_WS_STEPS_FP64])

    def samples_fp64(self):
        """In-snapshot samples taken near the hole in the last mixed-form
        launch (syncs)."""
        return int(self.ws[:32].cpu()[_lib.MK_WS_SAMPLES_FP64])

    def phase_b_work(self):
        """(steps, samples) the last MK_MIXED launch's near-hole kernel took
        (syncs)."""
        w = self.ws[:32].cpu()
        return int(w[_lib.MK_WS_STEPS_B]), int(w[_lib.MK_WS_SAMPLES_B])

    def phase_c_work(self):
        """(steps, samples) the last mixed-form launch's FP32 continuation
        kernel took (syncs)."""
        w = self.ws[:32].cpu()
        return int(w[_lib.MK_WS_STEPS_C]), int(w[_lib.MK_WS_SAMPLES_C])

    def zone_run_max(self):
        """Most steps one ray took in one visit to the mixed form's
        near-hole phase in the last launch (syncs): that phase's serial
        chain."""
        return int(self.ws[:32].cpu()[_lib.MK_WS_ZONE_RUN_MAX])

    def max_step_optical_depth(self):
        """Largest per-step w*alpha of the last launch (syncs); the explicit
        Euler transfer of the reference is stable while this stays below 1."""
        return float(self.ws[:32].cpu()[_lib.MK_WS_MAX_TAU:_lib.MK_WS_MAX_TAU + 1].view(torch.float64)[0])


def render_requests(requests, precision="fp64", stream=None, with_steps=False):
    """Render several requests in ONE persistent launch.

    Each request's ``out`` dict receives ``image`` ((nnu, res, res) float64
    CUDA tensor), ``check`` (PreparedRender.check of the launch: raises if
    a wait of the mixed form's near-hole pipeline ran out; syncs) and, with
    ``with_steps``, ``nsteps`` and ``status``.  Returns the list of image
    tensors.  The launch is asynchronous on ``stream`` (default: the current
    stream)."""
    if not requests:
        return []
    s = stream if stream is not None else torch.cuda.current_stream()
    with torch.cuda.stream(s):
        prep = PreparedRender(requests, precision, with_steps)
        images = prep.launch(s)
    # the request table and workspace stay alive until the launch retires
    for t in (prep.reqs_dev, prep.snaps_dev, prep.ws):
        t.record_stream(s)
    for r in requests:
        r.out["check"] = prep.check
    return images


def make_image(fluid_model, camera_inclination=60, camera_distance=1000, mass_scale=1.e26, M_bh=6.2e9 * Msun,
               r_high=40, observing_frequency=230.e9, fov=20, resolution=160, max_nsteps=10000,
               max_chunk_bytes=None, precision="fp64", r_low=1):
    """images.py:30-144 -> NumPy image (resolution, resolution) indexed [i_x, i_y];
    with a list of frequencies, (nnu, resolution, resolution)."""
    req = RenderRequest(fluid_model, camera_inclination, camera_distance, mass_scale, M_bh, r_high,
                        observing_frequency, fov, resolution, max_nsteps, r_low)
    s = torch.cuda.current_stream()
    with torch.cuda.stream(s):
        prep = PreparedRender([req], precision)
        img = prep.launch(s)[0]
        # the image and the launch's wait-error word come back into pinned
        # memory behind the render, then one synchronisation
        out_host = torch.empty(img.shape, dtype=img.dtype, pin_memory=True)
        out_host.copy_(img, non_blocking=True)
        err = torch.empty(1, dtype=torch.int64, pin_memory=True)
        err.copy_(prep.ws[_lib.MK_WS_ERROR:_lib.MK_WS_ERROR + 1], non_blocking=True)
    s.synchronize()
    if int(err[0]):
        raise _lib.MKError(_lib.MK_ERR_TIMEOUT, f"mk_render: {int(err[0])} waits of the near-hole pipeline ran out; "
                                                "the image is invalid")
    out = out_host.numpy()
    if np.ndim(observing_frequency) == 0:
        out = out[0]
    return out


def step_diagnostics(fluid_model, camera_inclination=60, camera_distance=1000, mass_scale=1.e26,
                     M_bh=6.2e9 * Msun, r_high=40, observing_frequency=230.e9, fov=20, resolution=160,
                     max_nsteps=10000, r_low=1):
    """make_image's per-step quantities from one fused FP64 launch.

    Returns a dict of CUDA tensors: ``em`` and ``ab`` (nnu, N_t, npx), the
    invariant emissivity and absorptivity at each trajectory row, ``dt``
    (N_t, npx), trimmed to the N_t rows geodesic_integrator keeps
    (geodesics.py:275-281); ``dIs`` (nnu, N_t - 1, npx), the per-step
    intensity changes solve_specific_intensity(dIs=True) returns
    (transfer.py:111-117, backward order), ``attenuated`` (nnu, N_t - 1,
    npx), solve_attenuated_emissivity (transfer.py:122-144); ``image``
    (nnu, res, res) and ``nsteps`` (res, res).  Rows after a ray stops hold
    zeros where the reference repeats the frozen state's sample; both carry
    dt = 0, so dIs and the attenuated emissivity agree there."""
    from .geodesics import trimmed_rows
    from .transfer import solve_attenuated_emissivity, solve_specific_intensity
    req = RenderRequest(fluid_model, camera_inclination, camera_distance, mass_scale, M_bh, r_high,
                        observing_frequency, fov, resolution, max_nsteps, r_low, rows=max_nsteps)
    PreparedRender([req], precision="fp64").launch()
    K = req.out["nsteps"].reshape(-1)
    nt = trimmed_rows(K, max_nsteps)
    em, ab, dt = req.out["rows_em"][:, :nt], req.out["rows_ab"][:, :nt], req.out["rows_dt"][:nt]
    L_unit = fluid_model.get_units(M_bh, mass_scale)["L_unit"]
    nnu = em.shape[0]
    dIs = torch.stack([solve_specific_intensity(em[c], ab[c], dt, L_unit, dIs=True)[1] for c in range(nnu)])
    att = torch.stack([solve_attenuated_emissivity(em[c], ab[c], dt, L_unit) for c in range(nnu)])
    return dict(image=req.out["image"], nsteps=req.out["nsteps"], em=em, ab=ab, dt=dt, dIs=dIs, attenuated=att)


def image_flux_jy(image, fov, distance_cm, L_unit):
    """Total flux (Jy) of an image of specific intensity: sum I dOmega with
    dOmega = (fov/res)^2 L_unit^2 / D^2 per pixel."""
    img = image.detach().cpu().numpy() if isinstance(image, torch.Tensor) else np.asarray(image)
    res = img.shape[-1]
    dpix = fov / res * L_unit / distance_cm
    return img.sum(axis=(-2, -1)) * dpix * dpix / JY
