"""Host-side API over libtm.so, mirroring the reference's interface.

Reference call shape (simulations/Percolation_FD/stochasticSPDP.cpp:940):

    percolationDornic_2D(Rho, t_meas, Rh0, t_max, a, b, D, sigma, dt, dx, r, g)

appends rows {a, L, t, <<rho>_x>_r, Var, #surviving runs, #active sites, #surv alt}
for t = 0, dt, ... <= 1 and for every t in t_meas.  `percolation_dornic_2d`
below takes the same arguments (plus a seed and a precision) and returns the
same rows, computed by one batched GPU run of all r replicates.
`critical_exp_delta` is the a-sweep around it (stochasticSPDP.cpp:1309-1422).
A `Batch` of `rietkerk_model()` runs the three-field Rietkerk step that
rietkerk_DorFPE_2D_MultiSp (rietkerk_bjork_FKE.cpp:3697) takes per time step;
`fke_advdiff` is that driver's consumer movement (advdiff_FKE_MultiSp).
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass, field

import numpy as np

from . import _lib as T


# ------------------------------------------------------------------ time grids
def linspace(start, end, num):
    """numpy-style linspace as the reference writes it (stochasticSPDP.cpp:254-279)."""
    if num == 0:
        return []
    if num == 1:
        return [float(start)]
    delta = (float(end) - float(start)) / (num - 1)
    return [float(start) + delta * i for i in range(num - 1)] + [float(end)]


def lnspace(start, end, num):
    """Natural-log-spaced points as the reference writes them (stochasticSPDP.cpp:281-301):
    e^(log start + i delta) for i < num - 1, then end exactly."""
    if num == 0:
        return []
    if num == 1:
        return [float(start)]
    lo, hi = math.log(float(start)), math.log(float(end))
    delta = (hi - lo) / (num - 1)
    base = math.exp(1)
    return [math.pow(base, lo + delta * i) for i in range(num - 1)] + [float(end)]


def logarithm10_time_bins(t_max: float, dt: float) -> list[float]:
    """Measurement times 10^0 .. 10^floor1(log10 t_max), 25 per decade, snapped
    down to the dt grid and de-duplicated (stochasticSPDP.cpp:336-378)."""
    out: list[float] = []
    if t_max <= 1:
        return out
    tend_one = math.floor(math.log10(t_max) * 10.0) / 10.0
    power = 0.0
    while power <= tend_one:
        t_raw = math.pow(10, power)
        q = t_raw / dt
        t_fin = float(int(q)) * dt  # static_cast<int>(t_raw/dt)*dt
        if t_fin <= 1.0:
            t_fin = t_fin + dt
        if len(out) > 0 and t_fin != out[-1]:
            out.append(t_fin)
        elif len(out) == 0:
            out.append(t_fin)
        power += 0.04
    for i in range(len(out) - 1, 0, -1):
        if out[i] < out[i - 1] + dt / 2.0:
            del out[i]
    return out


def reference_step_grid(t_meas, dt):
    """Step indices the reference measures at: every step while t <= 1 and then the
    step nearest each t in t_meas (stochasticSPDP.cpp:1003-1025, 1118-1122).
    Returns (steps, times, n_early) with n_early rows of the t <= 1 block."""
    times = []
    t = 0.0
    while t <= 1:
        times.append(t)
        t += dt
    n_early = len(times)
    times += [float(x) for x in t_meas]
    steps = [int(round(x / dt)) for x in times]
    return steps, times, n_early


# ------------------------------------------------------------------ context / batch
class Context:
    """A CUDA device plus a stream (tm_create)."""

    def __init__(self, device: int = 0):
        self._h = C.c_void_p()
        T.check(T.lib().tm_create(C.byref(self._h), device), "tm_create")
        self.device = device

    @property
    def handle(self):
        return self._h

    @property
    def stream(self) -> int:
        return int(T.lib().tm_stream(self._h) or 0)

    def sync(self):
        T.check(T.lib().tm_sync(self._h), "tm_sync")

    def set_test_probe(self, flags: int = 0):
        """Make a failure path run on purpose (TM_PROBE_*; tests only); 0 clears."""
        T.check(T.lib().tm_set_test_probe(self._h, int(flags)), "tm_set_test_probe")

    def close(self):
        if self._h:
            T.lib().tm_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:  # noqa: BLE001
            pass


def dp_model(b=2.0, c=0.0, D=1.0, sigma=1.0, dt=0.1, dx=1.0, clamp_lo=0.0, clamp_eps=0.0,
             remainder=T.TM_REM_EULER_EXACT, sampler=T.TM_SAMPLER_EXACT, deterministic=0, stencil=5,
             integrator=1) -> T.DPModel:
    return T.DPModel(b, c, D, sigma, dt, dx, clamp_lo, clamp_eps, remainder, sampler, deterministic, stencil,
                     integrator, 0)


def rietkerk_model(alpha=0.2, k2=5.0, W0=0.2, gmax=0.05, k1=5.0, c=10.0, d=0.25, rW=0.2, DP=0.1, DW=0.1, DO=100.0,
                   sigma=0.5, dt=1e-3, dx=1.0, clamp_lo=0.0, clamp_eps=1e-10, sampler=T.TM_SAMPLER_REF_GAUSS100,
                   deterministic=0) -> T.RietkerkModel:
    return T.RietkerkModel(alpha, k2, W0, gmax, k1, c, d, rW, DP, DW, DO, sigma, dt, dx, clamp_lo, clamp_eps, sampler,
                           deterministic)


def instances(Ls, seeds, a, a_step=0.0):
    n = len(Ls)
    a = np.broadcast_to(np.asarray(a, dtype=np.float64), (n,))
    a_step = np.broadcast_to(np.asarray(a_step, dtype=np.float64), (n,))
    arr = (T.Instance * n)()
    for k in range(n):
        arr[k] = T.Instance(int(Ls[k]), 0, int(seeds[k]) & 0xFFFFFFFFFFFFFFFF, float(a[k]), float(a_step[k]))
    return arr


def layout(inst, nf):
    n = len(inst)
    off = np.zeros(n, np.int64)
    fs = np.zeros(n, np.int64)
    total = T.lib().tm_layout(inst, n, nf, off.ctypes.data_as(C.POINTER(C.c_int64)),
                              fs.ctypes.data_as(C.POINTER(C.c_int64)))
    return int(total), off, fs


def pack(fields, inst, nf, dtype):
    """fields[k]: array (nf, L, L) or (L, L) -> packed 1-D buffer in the batch layout."""
    total, off, fs = layout(inst, nf)
    buf = np.zeros(total, dtype)
    for k, f in enumerate(fields):
        f = np.asarray(f, dtype).reshape(nf, -1)
        for j in range(nf):
            buf[off[k] + j * fs[k]: off[k] + j * fs[k] + f.shape[1]] = f[j]
    return buf


def unpack(buf, inst, nf):
    total, off, fs = layout(inst, nf)
    out = []
    for k in range(len(inst)):
        L = inst[k].L
        f = np.stack([buf[off[k] + j * fs[k]: off[k] + j * fs[k] + L * L].reshape(L, L) for j in range(nf)])
        out.append(f if nf > 1 else f[0])
    return out


class Batch:
    """A device-resident ragged batch of lattice instances (tm_batch_*)."""

    def __init__(self, ctx: Context, model, inst, precision=T.TM_FP64):
        self.ctx = ctx
        self.inst = inst
        self.n = len(inst)
        self.precision = precision
        self.dtype = np.float64 if precision == T.TM_FP64 else np.float32
        self._h = C.c_void_p()
        L = T.lib()
        if isinstance(model, T.DPModel):
            T.check(L.tm_batch_create_dp(ctx.handle, C.byref(model), inst, self.n, precision, C.byref(self._h)),
                    "tm_batch_create_dp")
        else:
            T.check(L.tm_batch_create_rietkerk(ctx.handle, C.byref(model), inst, self.n, precision,
                                               C.byref(self._h)), "tm_batch_create_rietkerk")
        self.nf = L.tm_batch_num_fields(self._h)
        self.obs_width = L.tm_batch_obs_width(self._h)
        self.total = int(L.tm_batch_total_elems(self._h))

    @property
    def handle(self):
        return self._h

    @property
    def step(self) -> int:
        return int(T.lib().tm_batch_step(self._h))

    def upload(self, fields, step=0):
        buf = np.ascontiguousarray(fields, self.dtype) if isinstance(fields, np.ndarray) and fields.ndim == 1 \
            else pack(fields, self.inst, self.nf, self.dtype)
        assert buf.size == self.total
        T.check(T.lib().tm_batch_upload(self._h, buf.ctypes.data_as(C.c_void_p), step), "tm_batch_upload")

    def upload_device(self, ptr: int, step=0):
        T.check(T.lib().tm_batch_upload_device(self._h, C.c_void_p(ptr), step), "tm_batch_upload_device")

    def download_packed(self):
        buf = np.empty(self.total, self.dtype)
        T.check(T.lib().tm_batch_download(self._h, buf.ctypes.data_as(C.c_void_p)), "tm_batch_download")
        return buf

    def download(self):
        return unpack(self.download_packed(), self.inst, self.nf)

    def snapshot(self, k):
        L = self.inst[k].L
        out = np.empty((self.nf, L, L), self.dtype)
        T.check(T.lib().tm_batch_snapshot(self._h, k, out.ctypes.data_as(C.c_void_p)), "tm_batch_snapshot")
        return out if self.nf > 1 else out[0]

    def advance(self, n_steps, meas_steps=()):
        ms = np.ascontiguousarray(meas_steps, np.int64)
        obs = np.zeros((max(len(ms), 1), self.n, self.obs_width))
        st = np.zeros(self.n, np.uint32)
        T.check(T.lib().tm_batch_advance(self._h, int(n_steps), ms.ctypes.data_as(C.POINTER(C.c_int64)), len(ms),
                                         obs.ctypes.data_as(C.POINTER(C.c_double)),
                                         st.ctypes.data_as(C.POINTER(C.c_uint32))), "tm_batch_advance")
        return obs[:len(ms)], st

    def enqueue_steps(self, n_steps):
        T.check(T.lib().tm_batch_enqueue_steps(self._h, int(n_steps)), "tm_batch_enqueue_steps")

    def set_launch(self, rows_per_task=0, ctas_per_sm=0):
        T.check(T.lib().tm_batch_set_launch(self._h, rows_per_task, ctas_per_sm), "tm_batch_set_launch")

    def get_launch(self):
        r, c = C.c_int(), C.c_int()
        T.check(T.lib().tm_batch_get_launch(self._h, C.byref(r), C.byref(c)), "tm_batch_get_launch")
        return r.value, c.value

    def autotune(self, steps_per_trial=4):
        T.check(T.lib().tm_batch_autotune(self._h, steps_per_trial), "tm_batch_autotune")
        return self.get_launch()

    def set_spreading(self, enable=True, cx=-1, cy=-1):
        """Spreading runs: measurements add the summed squared distance of occupied
        sites from the seed (obs width 3), and instances stop once activity reaches
        the lattice's edge (tm_batch_set_spreading)."""
        T.check(T.lib().tm_batch_set_spreading(self._h, int(enable), int(cx), int(cy)), "tm_batch_set_spreading")
        self.obs_width = T.lib().tm_batch_obs_width(self._h)

    def set_site_coeff(self, coeff):
        """Per-site loss coefficient b_v (list of (L, L) arrays or a packed buffer; None: uniform b)."""
        if coeff is None:
            T.check(T.lib().tm_batch_set_site_coeff(self._h, None), "tm_batch_set_site_coeff")
            return
        buf = np.ascontiguousarray(coeff, self.dtype) if isinstance(coeff, np.ndarray) and coeff.ndim == 1 \
            else pack(coeff, self.inst, self.nf, self.dtype)
        self._site_b = buf
        T.check(T.lib().tm_batch_set_site_coeff(self._h, buf.ctypes.data_as(C.c_void_p)), "tm_batch_set_site_coeff")

    def box_means(self, k, box, field=0):
        """Kadanoff block means (L/box x L/box) of instance k's field."""
        L = self.inst[k].L
        out = np.zeros((L // box) * (L // box))
        T.check(T.lib().tm_batch_box_means(self._h, k, field, box, out.ctypes.data_as(C.POINTER(C.c_double))),
                "tm_batch_box_means")
        return out.reshape(L // box, L // box)

    def power_spectrum(self, k, field=0, binwidth=0.5):
        """Radially averaged power spectrum of instance k's field (glow_up.py:752-827
        semantics); returns (kvals, power)."""
        L = self.inst[k].L
        cap = int(2 * L / binwidth) + 8
        kv = np.zeros(cap)
        pw = np.zeros(cap)
        nb = C.c_int()
        T.check(T.lib().tm_batch_power_spectrum(self._h, k, field, binwidth, kv.ctypes.data_as(C.POINTER(C.c_double)),
                                                pw.ctypes.data_as(C.POINTER(C.c_double)), cap, C.byref(nb)),
                "tm_batch_power_spectrum")
        return kv[:nb.value], pw[:nb.value]

    def close(self):
        if self._h:
            T.lib().tm_batch_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:  # noqa: BLE001
            pass


def pattern_wavelength(L, kvals, power):
    """Wavelength (lattice units) at the peak of a radial power spectrum: L / k_peak."""
    p = np.where(np.isfinite(power), power, -np.inf)
    return float(L) / float(kvals[int(np.argmax(p))])


# ------------------------------------------------------ consumer movement (FKE)
def _reference_pi():
    """The reference's PI: 15 terms of the Bailey-Borwein-Plouffe series summed
    from the smallest (CalculatePi<14>, rietkerk_bjork_basic.h:243-259, :284)."""
    s = 0.0
    for n in range(15):
        s = (1.0 / 16 ** n) * (4.0 / (8 * n + 1.0) - 2.0 / (8 * n + 4.0) - 1.0 / (8 * n + 5.0)
                               - 1.0 / (8 * n + 6.0)) + s
    return s


def gaussian_stencil(sigma, rbound):
    """precompute_gaussian (rietkerk_bjork_FKE.cpp:1735-1749): the one-sided
    Gaussian exp(-x^2 / 2 sigma^2) / (sqrt(2 pi) sigma) for x = 0..rbound,
    renormalised so that the two-sided stencil sums to 1."""
    factor = 1.0 / (math.sqrt(2 * _reference_pi()) * sigma)
    st = np.empty(rbound + 1)
    tot = 0.0
    for x in range(rbound + 1):
        st[x] = factor * math.exp(-0.5 * (x * x) / (sigma * sigma))
        tot += 2 * st[x] if x > 0 else st[0]
    return st / tot


@dataclass
class FKEParams:
    pref: float          # mu_vel_prefactor: shift = round(v * pref) lattice sites
    RD: int              # diffusion stencil bound (sites)
    RV: int              # advection stencil bound (sites)
    gD: np.ndarray       # diffusion stencil, RD + 1 values
    gV: np.ndarray       # advection stencil, RV + 1 values


def fke_parameters(D, v, dt_adv, sigma, dx=1.0, CI=4):
    """set_global_FKE_params (rietkerk_bjork_FKE.cpp:195-338, displacement-
    invariant default) for one consumer species: velocity relaxation beta =
    3 / dt_adv, diffusion width sqrt(2 D dt_adv), the OU displacement width of
    the velocity process, bounds int(CI * width / dx), and the shift prefactor
    (dt_adv - (1 - e^{-beta dt_adv}) / beta) / dx.  Both stencils are built with
    the species' `sigma`, as the reference's caller does (rietkerk_bjork_FKE.cpp:
    3764-3772)."""
    beta = 3.0 / dt_adv
    e1 = math.exp(-beta * dt_adv)
    e2 = math.exp(-2 * beta * dt_adv)
    sv = math.sqrt(2 * beta * 1 * abs(v))
    sigma_D = math.sqrt(2 * D * dt_adv)
    svx = (sv / beta) * math.sqrt(dt_adv + (1 / (2 * beta)) * (1 - e2) - (2 / beta) * (1 - e1))
    RD = int(CI * sigma_D / dx)
    RV = int(CI * svx / dx)
    pref = (1 / dx) * (dt_adv - ((1 - e1) / beta))
    return FKEParams(pref, RD, RV, gaussian_stencil(sigma, RD), gaussian_stencil(sigma, RV))


def fke_workspace(L, precision=T.TM_FP64, device=0):
    """A device workspace for fke_advdiff(..., workspace=...) on L x L lattices
    (tm_fke_workspace_bytes), allocated by torch, reusable for every step."""
    import torch
    n = int(T.lib().tm_fke_workspace_bytes(precision, int(L)))
    if n == 0:
        raise T.TMError(T.TM_ERR_INVALID, "fke_workspace: precision or L")
    return torch.empty(n + 256, dtype=torch.uint8, device=torch.device("cuda", device))


def fke_advdiff(rho, gamma, vx, vy, params: FKEParams, eps=1e-10, precision=T.TM_FP64, device=0, workspace=None):
    """One FKE advection-diffusion of a consumer field (advdiff_FKE_MultiSp,
    rietkerk_bjork_FKE.cpp:3614-3695) through tm_fke_advdiff_device.  rho, gamma,
    vx, vy are L x L arrays (numpy, or CUDA torch tensors of the precision's
    dtype, which are used in place); returns the moved field in the same kind.
    With workspace (fke_workspace) the call goes through tm_fke_advdiff_device_ws:
    no allocation and no synchronisation inside the library (torch tensors in,
    a torch tensor out, ready on the current stream)."""
    import torch
    dt = torch.float64 if precision == T.TM_FP64 else torch.float32
    as_numpy = isinstance(rho, np.ndarray)
    dev = torch.device("cuda", device)
    ts = [torch.as_tensor(np.ascontiguousarray(a), dtype=dt).to(dev) if as_numpy else a.contiguous()
          for a in (rho, gamma, vx, vy)]
    L = ts[0].shape[0]
    if any(t.shape != (L, L) or t.dtype != dt or t.device != dev for t in ts):
        raise T.TMError(T.TM_ERR_INVALID, "fke_advdiff: four L x L fields of one dtype on one device")
    out = torch.empty_like(ts[0])
    gD = np.ascontiguousarray(params.gD, np.float64)
    gV = np.ascontiguousarray(params.gV, np.float64)
    with torch.cuda.device(dev):
        s = torch.cuda.current_stream(dev)
        args = (*(t.data_ptr() for t in ts), precision, L, params.pref, eps,
                gD.ctypes.data_as(C.POINTER(C.c_double)), len(gD) - 1, gV.ctypes.data_as(C.POINTER(C.c_double)),
                len(gV) - 1, out.data_ptr())
        if workspace is None:
            T.check(T.lib().tm_fke_advdiff_device(*args, s.cuda_stream), "tm_fke_advdiff_device")
        else:
            base = workspace.data_ptr()
            aligned = (base + 255) // 256 * 256
            T.check(T.lib().tm_fke_advdiff_device_ws(*args, aligned, workspace.numel() - (aligned - base),
                                                     s.cuda_stream), "tm_fke_advdiff_device_ws")
    return out.cpu().numpy() if as_numpy else out


def run_dp(ctx, model, inst, init_packed, n_steps, meas_steps, precision):
    """tm_run_dp: host buffers in, observables/status/final fields out."""
    ms = np.ascontiguousarray(meas_steps, np.int64)
    n = len(inst)
    init = np.ascontiguousarray(init_packed)
    obs = np.zeros((max(len(ms), 1), n, 2))
    st = np.zeros(n, np.uint32)
    fin = np.empty_like(init)
    T.check(T.lib().tm_run_dp(ctx.handle, C.byref(model), inst, n, precision, init.ctypes.data_as(C.c_void_p),
                              int(n_steps), ms.ctypes.data_as(C.POINTER(C.c_int64)), len(ms),
                              obs.ctypes.data_as(C.POINTER(C.c_double)), st.ctypes.data_as(C.POINTER(C.c_uint32)),
                              fin.ctypes.data_as(C.c_void_p)), "tm_run_dp")
    return obs[:len(ms)], st, fin


# ------------------------------------------------------------------ reference-shaped calls
def replicate_rows(a, L, times, n_early, mean, active):
    """Rows {a, L, t, <<rho>_x>_r, Var, #surviving, <#active>_surv, surv_alt} from per-replicate
    series mean[j, i], active[j, i] (stochasticSPDP.cpp:1078-1142).  The variance is the
    unbiased sample variance over the surviving replicates (the reference's running
    formula divides by (1/(r-1)) in integer arithmetic, :202, so its column is not used)."""
    r = mean.shape[0]
    rows = []
    for i, t in enumerate(times):
        alive = active[:, i] > 0
        ns = int(alive.sum())
        mu = float(mean[alive, i].mean()) if ns else 0.0
        var = float(mean[alive, i].var(ddof=1)) if ns > 1 else 0.0
        act = float(active[alive, i].mean()) if ns else 0.0
        alt = float(r) if i < n_early else float(ns)
        rows.append([a, float(L), float(t), mu, var, float(ns), act, alt])
    return np.array(rows)


def percolation_dornic_2d(t_meas, Rh0, t_max, a, b, D, sigma, dt, dx, r, g, *, seed=0, precision=T.TM_FP64,
                          ctx: Context | None = None, a_end=None, remainder=T.TM_REM_EULER_EXACT,
                          sampler=T.TM_SAMPLER_EXACT, clamp_lo=0.0, clamp_eps=0.0, c=0.0):
    """GPU percolationDornic_2D: r replicates of one g x g lattice, returned as the
    reference's rows.  Replicate j uses Philox key seed + j (the reference seeds
    std::mt19937_64 with random_device()+j, :973-976).  a_end gives a linear ramp
    of a over the run (a(s) = a + (a_end - a) s / n_steps)."""
    ctx = ctx or Context(0)
    steps, times, n_early = reference_step_grid(t_meas, dt)
    n_steps = max(steps)
    a_step = 0.0 if a_end is None else (a_end - a) / float(n_steps)
    inst = instances([g] * r, [seed + j for j in range(r)], a, a_step)
    model = dp_model(b=b, c=c, D=D, sigma=sigma, dt=dt, dx=dx, clamp_lo=clamp_lo, clamp_eps=clamp_eps,
                     remainder=remainder, sampler=sampler)
    dtype = np.float64 if precision == T.TM_FP64 else np.float32
    init = pack([np.asarray(Rh0, np.float64).reshape(g, g)] * r, inst, 1, dtype)
    obs, st, _ = run_dp(ctx, model, inst, init, n_steps, steps, precision)
    mean = obs[:, :, 0].T.copy()
    act = obs[:, :, 1].T.copy()
    return replicate_rows(a, g, times, n_early, mean, act), st


def shard_indices(n, rank, world):
    """The contiguous block of range(n) that one of `world` ranks takes (the first
    n % world ranks take one more): the static split of a sweep's control values."""
    base, extra = divmod(int(n), int(world))
    start = rank * base + min(rank, extra)
    return list(range(start, start + base + (1 if rank < extra else 0)))


def _sweep_block(ctx, indices, avals, Rho_0, t_max, b, D, sigma, dt, dx, r, g, seed, precision):
    """Rows and status of the control values `indices` of a sweep, in one batch:
    {index: (rows, status of its r replicates)}.  Replicate j of value i has the
    Philox key seed + i r + j whichever rank runs it."""
    if not indices:
        return {}
    t_meas = logarithm10_time_bins(t_max, dt)
    steps, times, n_early = reference_step_grid(t_meas, dt)
    Ls, seeds, av = [], [], []
    for ia in indices:
        for j in range(r):
            Ls.append(g); seeds.append(seed + ia * r + j); av.append(avals[ia])
    inst = instances(Ls, seeds, av)
    model = dp_model(b=b, D=D, sigma=sigma, dt=dt, dx=dx)
    dtype = np.float64 if precision == T.TM_FP64 else np.float32
    init = pack([np.asarray(Rho_0, np.float64).reshape(g, g)] * len(Ls), inst, 1, dtype)
    obs, st, _ = run_dp(ctx, model, inst, init, max(steps), steps, precision)
    out = {}
    for k, ia in enumerate(indices):
        sl = slice(k * r, (k + 1) * r)
        out[ia] = (replicate_rows(avals[ia], g, times, n_early, obs[:, sl, 0].T, obs[:, sl, 1].T), st[sl])
    return out


def gather_blocks(blocks, rank, world):
    """Every rank's {index: ...} blocks merged on rank 0 (a host gather over the
    initialised torch.distributed group); None on the other ranks."""
    if world == 1:
        return dict(blocks)
    import torch.distributed as dist
    got = [None] * world if rank == 0 else None
    dist.gather_object(blocks, got, dst=0)
    if rank != 0:
        return None
    merged = {}
    for part in got:
        merged.update(part)
    return merged


def critical_exp_delta(Rho_0, div, t_max, a_start, a_end, b, D, sigma, dt, dx, r, g, *, seed=0,
                       precision=T.TM_FP64, ctx: Context | None = None, distributed=False):
    """The a-sweep of stochasticSPDP.cpp:1309-1422 in one batch: div values of a
    (linspace), r replicates each, rows concatenated in a order.

    distributed=True splits the a-values over the ranks of the initialised
    torch.distributed group (one GPU each): every rank runs its contiguous block
    as one batch, and rank 0 gathers the rows on the host and returns the same
    rows as a single-GPU run (the replicates' keys do not depend on the split);
    the other ranks return (None, None)."""
    ctx = ctx or Context(0)
    avals = linspace(a_start, a_end, div)
    if distributed:
        import torch.distributed as dist
        rank, world = dist.get_rank(), dist.get_world_size()
    else:
        rank, world = 0, 1
    mine = shard_indices(div, rank, world)
    blocks = _sweep_block(ctx, mine, avals, Rho_0, t_max, b, D, sigma, dt, dx, r, g, seed, precision)
    merged = gather_blocks(blocks, rank, world)
    if merged is None:
        return None, None
    return (np.concatenate([merged[ia][0] for ia in range(div)]),
            np.concatenate([merged[ia][1] for ia in range(div)]))

# ------------------------------------------------------ finite-size and spreading sweeps
def init_fullframe(g):
    """Every site at 1 (init_fullframe, stochasticSPDP.cpp:39-44)."""
    return np.ones(g * g)


def init_solitarytear(g):
    """A single occupied site at (int(g/2), int(g/2)) (init_solitarytear, stochasticSPDP.cpp:88-95)."""
    a = np.zeros(g * g)
    h = int(g / 2.0)
    a[g * h + h] = 1.0
    return a


def _ragged_dp_rows(ctx, groups, t_meas, t_max, a, b, D, sigma, dt, dx, r, seed, precision):
    """One batch for several lattice sizes: groups = [(L, init frame)], r replicates each,
    measured on one grid; returns [(L, rows, status)] in group order.  Replicate j of
    group i has the Philox key seed + i r + j."""
    steps, times, n_early = reference_step_grid(t_meas, dt)
    Ls, seeds = [], []
    for i, (L, _) in enumerate(groups):
        for j in range(r):
            Ls.append(L); seeds.append(seed + i * r + j)
    inst = instances(Ls, seeds, a)
    model = dp_model(b=b, D=D, sigma=sigma, dt=dt, dx=dx)
    dtype = np.float64 if precision == T.TM_FP64 else np.float32
    init = pack([np.asarray(f, np.float64).reshape(L, L) for L, f in groups for _ in range(r)], inst, 1, dtype)
    obs, st, _ = run_dp(ctx, model, inst, init, max(steps), steps, precision)
    out = []
    for i, (L, _) in enumerate(groups):
        sl = slice(i * r, (i + 1) * r)
        out.append((L, replicate_rows(a, L, times, n_early, obs[:, sl, 0].T, obs[:, sl, 1].T), st[sl]))
    return out


def critical_exp_finite_scaling_collapse(div, g_st, g_end, t_max, a_c, b, D, sigma, dt, dx, r, *, seed=0,
                                         precision=T.TM_FP64, ctx: Context | None = None):
    """The finite-size sweep of stochasticSPDP.cpp:1424-1536 at a_c: lattice sides
    int(linspace(g_st, g_end, div)), r replicates each from a full frame, measured on
    logarithm10_time_bins(t_max, dt); every side in one ragged batch.  Returns the
    reference's rows {a, L, t, <<rho>_x>_r, Var, #surviving, #active, surv-alt} in
    side order, and the replicates' status bits."""
    ctx = ctx or Context(0)
    g_space = [int(g) for g in linspace(g_st, g_end, div)]
    res = _ragged_dp_rows(ctx, [(g, init_fullframe(g)) for g in g_space], logarithm10_time_bins(t_max, dt), t_max,
                          a_c, b, D, sigma, dt, dx, r, seed, precision)
    return np.concatenate([rows for _, rows, _ in res]), np.concatenate([st for _, _, st in res])


def stationary_window(g):
    """Measurement window (t_start, t_end) of the stationary finite-size sweep for side g
    (stochasticSPDP.cpp:1600-1610).  The reference sets none for g <= 30 (its values are
    then uninitialised), so such sides are rejected."""
    if 30 < g <= 50:
        return 300.0, 900.0
    if 50 < g <= 100:
        return 1000.0, 2500.0
    if 100 < g <= 150:
        return 1250.0, 8000.0
    if 150 < g <= 200:
        return 1400.0, 10000.0
    if g > 200:
        return 2000.0, 15000.0
    raise ValueError(f"critical_exp_finite_scaling_stationary: no measurement window for L = {g} <= 30")


def critical_exp_finite_scaling_stationary(div, g_st, g_end, t_lim, t_max, a_c, b, D, sigma, dt, dx, r, *, seed=0,
                                           precision=T.TM_FP64, ctx: Context | None = None):
    """The stationary finite-size sweep of stochasticSPDP.cpp:1539-1670 at a_c: sides
    int(lnspace(g_st, g_end, div)), r replicates each from a full frame, each side
    measured at linspace(t_start, t_end, 30) of its window (stationary_window).
    Sides sharing a window run as one ragged batch.  t_lim and t_max are accepted
    for the reference's argument order; the reference's runs end at t_end + 10,
    after their last measurement, so they do not change the rows.  Returns rows in
    side order and the replicates' status bits."""
    ctx = ctx or Context(0)
    g_space = [int(g) for g in lnspace(g_st, g_end, div)]
    windows = [stationary_window(g) for g in g_space]
    by_window = {}
    for i, (g, w) in enumerate(zip(g_space, windows)):
        by_window.setdefault(w, []).append(i)
    per_side = {}
    for w, idx in by_window.items():
        t_meas = linspace(w[0], w[1], 30)
        res = _ragged_dp_rows(ctx, [(g_space[i], init_fullframe(g_space[i])) for i in idx], t_meas, w[1] + 10,
                              a_c, b, D, sigma, dt, dx, r, seed + 7919 * min(idx), precision)
        for i, (_, rows, st) in zip(idx, res):
            per_side[i] = (rows, st)
    return (np.concatenate([per_side[i][0] for i in range(len(g_space))]),
            np.concatenate([per_side[i][1] for i in range(len(g_space))]))


def spreading_rows(block, a, times, n_active, sq_dist):
    """Rows {block, a, t, <N(t)>_r, <MSD(t)>_r, #surviving} of spreading runs from
    per-replicate series n_active[j, i] (occupied sites) and sq_dist[j, i] (summed
    squared distance): means over the replicates still running at t
    (spreading_incremental_surv_runs, stochasticSPDP.cpp:230-252; the reference's
    first column is the OpenMP thread, here the block index)."""
    rows = []
    for i, t in enumerate(times):
        alive = n_active[:, i] > 0
        ns = int(alive.sum())
        N = float(n_active[alive, i].mean()) if ns else 0.0
        msd = float((sq_dist[alive, i] / n_active[alive, i]).mean()) if ns else 0.0
        rows.append([float(block), a, float(t), N, msd, float(ns)])
    return np.array(rows)


def critical_exp_theta_delta(Rho_0, div, t_max, a_c, b, D, sigma, dt, dx, r, g, *, seed=0, precision=T.TM_FP64,
                             ctx: Context | None = None):
    """Spreading experiments of stochasticSPDP.cpp:1673-1764: div blocks of r
    replicates started from a single seed at the centre (init_solitarytear; Rho_0 is
    ignored, as in the reference, which overwrites it), each measuring the number of
    occupied sites N(t) and their mean squared distance from the seed on
    logarithm10_time_bins(t_max, dt), and stopping once activity reaches the edge
    (spreading_exp_Dornic_2D, :1145-1298).  All div x r replicates run as one batch.
    Returns rows {block, a, t, <N>_r, <MSD>_r, #surviving} in block order, and the
    replicates' status bits."""
    ctx = ctx or Context(0)
    t_meas = logarithm10_time_bins(t_max, dt)
    steps, times, _ = reference_step_grid(t_meas, dt)
    n = div * r
    inst = instances([g] * n, [seed + j for j in range(n)], a_c)
    dtype = np.float64 if precision == T.TM_FP64 else np.float32
    bt = Batch(ctx, dp_model(b=b, D=D, sigma=sigma, dt=dt, dx=dx), inst, precision)
    try:
        bt.set_spreading(True)
        bt.upload([init_solitarytear(g).reshape(g, g).astype(dtype)] * n)
        obs, st = bt.advance(max(steps), steps)
    finally:
        bt.close()
    rows = [spreading_rows(i, a_c, times, obs[:, i * r:(i + 1) * r, 1].T, obs[:, i * r:(i + 1) * r, 2].T)
            for i in range(div)]
    return np.concatenate(rows), st
