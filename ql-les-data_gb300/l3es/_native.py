"""ctypes binding of the l3es_gb300 C ABI (include/l3es_gb300.h).

The library is built in tree by ``ql-les-data_gb300/build.py`` (or
``__graft_entry__.build()``). There is no fallback: if the library is missing,
importing this module raises with the build command, and every call checks the
returned status and raises ``RuntimeError`` with ``l3es_last_error()``.
Tensors are torch CUDA tensors; only their device pointers cross the boundary.
"""

from __future__ import annotations

import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(os.path.dirname(HERE), "lib", "libl3es_gb300.so")

FORCING = {"none": 0, "ekin_tot": 1, "const_power": 2}

# Every symbol declared in include/l3es_gb300.h: (restype, argtypes)
_P = ctypes.c_void_p
_I = ctypes.c_int32
_SIGNATURES = {
    "l3es_plan_create": (ctypes.c_int, [_P, ctypes.POINTER(_P)]),
    "l3es_plan_destroy": (ctypes.c_int, [_P]),
    "l3es_plan_check": (ctypes.c_int, [_P]),
    "l3es_selftest_bounded_wait": (ctypes.c_int, [_P]),
    "l3es_plan_set_e0": (ctypes.c_int, [_P, _P, _I]),
    "l3es_plan_workspace_bytes": (ctypes.c_int64, [_P]),
    "l3es_plan_set_nu": (ctypes.c_int, [_P, _P, _I]),
    "l3es_plan_get_schedule": (ctypes.c_int, [_P, _P]),
    "l3es_plan_set_schedule": (ctypes.c_int, [_P, _P]),
    "l3es_plan_get_step_form": (ctypes.c_int, [_P, _P]),
    "l3es_plan_set_step_form": (ctypes.c_int, [_P, ctypes.c_int32]),
    "l3es_plan_autotune": (ctypes.c_int, [_P, ctypes.c_char_p, _P]),
    "l3es_graph_begin": (ctypes.c_int, [ctypes.POINTER(_P)]),
    "l3es_graph_end": (ctypes.c_int, [_P, ctypes.POINTER(_P)]),
    "l3es_graph_launch": (ctypes.c_int, [_P, _P]),
    "l3es_graph_fork": (ctypes.c_int, [_P, ctypes.POINTER(_P)]),
    "l3es_graph_join": (ctypes.c_int, [_P, _P]),
    "l3es_graph_destroy": (ctypes.c_int, [_P]),
    "l3es_step": (ctypes.c_int, [_P, _P, _P, _I, _P, _P]),
    "l3es_step_energy": (ctypes.c_int, [_P, _P, _P, _I, _P, _P, _P]),
    "l3es_rhs": (ctypes.c_int, [_P, _P, _P, _P]),
    "l3es_rfftn": (ctypes.c_int, [_P, _P, _P, _P]),
    "l3es_irfftn": (ctypes.c_int, [_P, _P, _P, _P]),
    "l3es_kinetic_energy": (ctypes.c_int, [_P, _P, _P, _P]),
    "l3es_field_stats": (ctypes.c_int, [_P, _P, _P, _P]),
    "l3es_dissipation": (ctypes.c_int, [_P, _P, ctypes.c_double, _P, _P]),
    "l3es_energy_spectrum": (ctypes.c_int, [_P, _P, ctypes.c_double, _P, _P]),
    "l3es_plan_timing": (ctypes.c_int, [_P, _I]),
    "l3es_plan_kernel_stats": (ctypes.c_int, [_P, _I, ctypes.POINTER(ctypes.c_double),
                                              ctypes.POINTER(ctypes.c_int64),
                                              ctypes.POINTER(ctypes.c_double)]),
    "l3es_kernel_kind_count": (ctypes.c_int32, []),
    "l3es_kernel_kind_name": (ctypes.c_char_p, [_I]),
    "l3es_interp_plan_create": (ctypes.c_int, [_I, _I, _I, _I, ctypes.c_int64, ctypes.POINTER(_P)]),
    "l3es_interp_plan_create_batch": (ctypes.c_int, [_I, _I, _I, _I, ctypes.c_int64, _I, ctypes.POINTER(_P)]),
    "l3es_interp_plan_destroy": (ctypes.c_int, [_P]),
    "l3es_interp_set_spectrum": (ctypes.c_int, [_P, _P, _P]),
    "l3es_interp_set_field": (ctypes.c_int, [_P, _P, _P]),
    "l3es_interp_coarse_field": (ctypes.c_int, [_P, _P, _P]),
    "l3es_interp_coarse_spectrum": (ctypes.c_int, [_P, _P, _P]),
    "l3es_interp": (ctypes.c_int, [_P, _P, ctypes.c_int64, _P, _I, ctypes.c_double, _P, _P]),
    "l3es_interp_advect_rk4": (ctypes.c_int, [_P, _P, ctypes.c_int64, _P, _I, ctypes.c_double, _P, _P]),
    "l3es_interp_vjp": (ctypes.c_int, [_P, _P, ctypes.c_int64, _P, _I, _P, _P]),
    "l3es_shift": (ctypes.c_int, [_P, _P, ctypes.c_int64, ctypes.c_double, ctypes.c_double, _P, _P]),
    "l3es_interp_particles_to_grid": (ctypes.c_int, [_P, _P, _P, ctypes.c_int64, _P, _P]),
    "l3es_interp_dft_noalloc": (ctypes.c_int, [_I, _I, _I, _P, _P, ctypes.c_int64, _P, _P]),
    "l3es_plan_adjoint_prepare": (ctypes.c_int, [_P]),
    "l3es_rhs_vjp": (ctypes.c_int, [_P, _P, _P, _P, _P]),
    "l3es_adjoint_step": (ctypes.c_int, [_P, _P, _P, _P]),
    "l3es_interp_coarse_mse": (ctypes.c_int, [_P, _P, _P, _P, _P, _P]),
    "l3es_sph_plan_create": (ctypes.c_int, [_I, _I, ctypes.c_double, ctypes.c_int64, ctypes.POINTER(_P)]),
    "l3es_sph_plan_destroy": (ctypes.c_int, [_P]),
    "l3es_sph_density": (ctypes.c_int, [_P, _P, ctypes.c_int64, _P, _P]),
    "l3es_sph_relax_acceleration": (ctypes.c_int, [_P, _P, ctypes.c_int64, ctypes.c_double, _P, _P]),
    "l3es_sph_forces": (ctypes.c_int, [_P, _P, _P, ctypes.c_int64, ctypes.c_double, _P, _P, _P, _P]),
    "l3es_sph_relax_velocity": (ctypes.c_int, [_P, _P, _P, ctypes.c_int64, ctypes.c_double, ctypes.c_double,
                                               ctypes.c_double, _P, _P, _P]),
    "l3es_last_error": (ctypes.c_char_p, []),
    "l3es_version": (ctypes.c_char_p, []),
}


class PlanDesc(ctypes.Structure):
    """l3es_plan_desc."""

    _fields_ = [
        ("dim", ctypes.c_int32),
        ("n", ctypes.c_int32),
        ("batch", ctypes.c_int32),
        ("forcing", ctypes.c_int32),
        ("kf", ctypes.c_int32),
        ("kolm_k", ctypes.c_int32),
        ("nu", ctypes.c_double),
        ("dt", ctypes.c_double),
        ("e_kin_init", ctypes.c_double),
        ("eps_inj", ctypes.c_double),
        ("drag", ctypes.c_double),
        ("kolm_amp", ctypes.c_double),
        ("scheme", ctypes.c_int32),
    ]


# l3es_plan_desc.scheme: the reference's explicit viscous term, or the integrating factor
SCHEMES = {"explicit": 0, "integrating_factor": 1}


_lib = None


def load(path: str = LIB_PATH) -> ctypes.CDLL:
    """Load the library once (raises ImportError if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise ImportError(
            f"l3es_gb300 CUDA library not found at {path}; build it with "
            "`python ql-les-data_gb300/build.py` (nvcc, sm_103a)"
        )
    lib = ctypes.CDLL(path)
    for name, (res, args) in _SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


ENONFINITE = -6  # L3ES_ENONFINITE


class NonFiniteError(RuntimeError):
    """A step wrote NaN or infinite values into the state (the flow blew up)."""


def _check(rc: int, what: str) -> None:
    if rc != 0:
        msg = load().l3es_last_error().decode()
        cls = NonFiniteError if rc == ENONFINITE else RuntimeError
        raise cls(f"{what} failed ({rc}): {msg}")


def _stream(stream=None) -> int:
    import torch

    s = stream if stream is not None else torch.cuda.current_stream()
    return s.cuda_stream


def _ptr(t) -> int:
    if t is None:
        return None
    if not t.is_cuda:
        raise ValueError("l3es_gb300 calls need CUDA tensors")
    if not t.is_contiguous():
        raise ValueError("l3es_gb300 calls need contiguous tensors")
    return t.data_ptr()


class Plan:
    """Owns an ``l3es_plan``: twiddles, dealias band and scratch of one solver."""

    def __init__(self, dim: int, n: int, nu: float, dt: float, batch: int = 1,
                 forcing: str = "none", kf: int = 0, e_kin_init: float = 0.0,
                 eps_inj: float = 0.0, drag: float = 0.0, kolm_k: int = 0,
                 kolm_amp: float = 0.0, scheme: str = "explicit"):
        lib = load()
        if forcing not in FORCING:
            raise ValueError(f"forcing must be one of {list(FORCING)}, got {forcing!r}")
        if scheme not in SCHEMES:
            raise ValueError(f"scheme must be one of {list(SCHEMES)}, got {scheme!r}")
        self.dim, self.n, self.batch = int(dim), int(n), int(batch)
        self.nu, self.dt = float(nu), float(dt)
        self.forcing, self.kf, self.scheme = forcing, int(kf or 0), scheme
        d = PlanDesc(self.dim, self.n, self.batch, FORCING[forcing], self.kf, int(kolm_k),
                     self.nu, self.dt, float(e_kin_init), float(eps_inj), float(drag),
                     float(kolm_amp), SCHEMES[scheme])
        h = ctypes.c_void_p()
        _check(lib.l3es_plan_create(ctypes.byref(d), ctypes.byref(h)), "l3es_plan_create")
        self._h = h
        self._lib = lib

    # shapes -------------------------------------------------------------------
    @property
    def spec_shape(self):
        n, h = self.n, self.n // 2 + 1
        s = (3, n, n, h) if self.dim == 3 else (3, n, h)
        return s if self.batch == 1 else (self.batch,) + s

    @property
    def phys_shape(self):
        n = self.n
        s = (3, n, n, n) if self.dim == 3 else (3, n, n, 1)
        return s if self.batch == 1 else (self.batch,) + s

    def _check_spec(self, t):
        import torch

        if t.dtype != torch.complex64 or tuple(t.shape) != self.spec_shape:
            raise ValueError(f"expected complex64 {self.spec_shape}, got {t.dtype} {tuple(t.shape)}")
        if not t.is_contiguous() or t.data_ptr() % 16:
            raise ValueError("spectra must be contiguous and 16-byte aligned (the kernels read two modes at a time)")

    def _check_phys(self, t):
        import torch

        if t.dtype != torch.float32 or t.numel() != _prod(self.phys_shape):
            raise ValueError(f"expected float32 {self.phys_shape}, got {t.dtype} {tuple(t.shape)}")

    # calls --------------------------------------------------------------------
    def set_e0(self, e0) -> None:
        vals = (ctypes.c_double * self.batch)(*[float(v) for v in (e0 if hasattr(e0, "__len__") else [e0] * self.batch)])
        _check(self._lib.l3es_plan_set_e0(self._h, vals, self.batch), "l3es_plan_set_e0")

    def set_nu(self, nu) -> None:
        """Per-trajectory viscosities (one value per batch member)."""
        vals = (ctypes.c_double * self.batch)(*[float(v) for v in (nu if hasattr(nu, "__len__") else [nu] * self.batch)])
        _check(self._lib.l3es_plan_set_nu(self._h, vals, self.batch), "l3es_plan_set_nu")

    def step(self, u_hat, nsteps: int = 1, u_out=None, e_inj=None, ke=None, stream=None) -> None:
        """In-place RK4 steps on u_hat (optionally irfftn into u_out at the end). ke: a
        float64 device tensor of `batch` values that receives the kinetic energy of the
        final state (one float-float energy pass over it, inside the same call)."""
        self._check_spec(u_hat)
        if u_out is not None:
            self._check_phys(u_out)
        if ke is None:
            _check(self._lib.l3es_step(self._h, _ptr(u_hat), _ptr(u_out), int(nsteps), _ptr(e_inj),
                                       _stream(stream)), "l3es_step")
            return
        import torch

        if ke.dtype != torch.float64 or ke.numel() < self.batch:
            raise ValueError("ke must hold `batch` float64 values")
        _check(self._lib.l3es_step_energy(self._h, _ptr(u_hat), _ptr(u_out), int(nsteps), _ptr(e_inj), _ptr(ke),
                                          _stream(stream)), "l3es_step_energy")

    def rhs(self, u_hat, du, stream=None) -> None:
        self._check_spec(u_hat)
        self._check_spec(du)
        _check(self._lib.l3es_rhs(self._h, _ptr(u_hat), _ptr(du), _stream(stream)), "l3es_rhs")

    def adjoint_prepare(self) -> None:
        """Allocate the adjoint workspace now (before any stream capture)."""
        _check(self._lib.l3es_plan_adjoint_prepare(self._h), "l3es_plan_adjoint_prepare")

    def rhs_vjp(self, u_hat, g, out, stream=None) -> None:
        """out = (d rhs / d u_hat)^T g (gradient convention dL/dRe + i dL/dIm)."""
        self._check_spec(u_hat)
        self._check_spec(g)
        self._check_spec(out)
        _check(self._lib.l3es_rhs_vjp(self._h, _ptr(u_hat), _ptr(g), _ptr(out), _stream(stream)), "l3es_rhs_vjp")

    def adjoint_step(self, u_hat_n, lam, stream=None) -> None:
        """lam <- (d step / d u_hat_n)^T lam for one RK4 step from the checkpoint u_hat_n."""
        self._check_spec(u_hat_n)
        self._check_spec(lam)
        _check(self._lib.l3es_adjoint_step(self._h, _ptr(u_hat_n), _ptr(lam), _stream(stream)),
               "l3es_adjoint_step")

    def rfftn(self, u, u_hat, stream=None) -> None:
        self._check_phys(u)
        self._check_spec(u_hat)
        _check(self._lib.l3es_rfftn(self._h, _ptr(u), _ptr(u_hat), _stream(stream)), "l3es_rfftn")

    def irfftn(self, u_hat, u, stream=None) -> None:
        self._check_spec(u_hat)
        self._check_phys(u)
        _check(self._lib.l3es_irfftn(self._h, _ptr(u_hat), _ptr(u), _stream(stream)), "l3es_irfftn")

    def check(self) -> None:
        """Synchronises and raises if one of this plan's kernels gave up a bounded wait
        on its bulk copies since the last check (RuntimeError: the results of that call
        are invalid), or if a step wrote NaN or infinite values into the state
        (NonFiniteError: the flow blew up). Clears the flags."""
        _check(self._lib.l3es_plan_check(self._h), "l3es_plan_check")

    def kinetic_energy(self, u_hat, out, stream=None) -> None:
        self._check_spec(u_hat)
        _check(self._lib.l3es_kinetic_energy(self._h, _ptr(u_hat), _ptr(out), _stream(stream)),
               "l3es_kinetic_energy")

    def field_stats(self, u, out, stream=None) -> None:
        """out (float64, 4 per trajectory): max|u_x|, max|u_y|, max|u_z|, kinetic energy."""
        self._check_phys(u)
        _check(self._lib.l3es_field_stats(self._h, _ptr(u), _ptr(out), _stream(stream)), "l3es_field_stats")

    def dissipation(self, u_hat, nu, out, stream=None) -> None:
        self._check_spec(u_hat)
        _check(self._lib.l3es_dissipation(self._h, _ptr(u_hat), float(nu), _ptr(out), _stream(stream)),
               "l3es_dissipation")

    def energy_spectrum(self, u_hat, out, mul_fac: float = 1.0, stream=None) -> None:
        self._check_spec(u_hat)
        _check(self._lib.l3es_energy_spectrum(self._h, _ptr(u_hat), float(mul_fac), _ptr(out), _stream(stream)),
               "l3es_energy_spectrum")

    def timing(self, enable: bool) -> None:
        """Start (clearing the counters) or stop per-launch CUDA-event timing."""
        _check(self._lib.l3es_plan_timing(self._h, int(bool(enable))), "l3es_plan_timing")

    def kernel_stats(self) -> dict:
        """{kernel name: (launches, total ms, algorithmic bytes)} since timing(True)."""
        out = {}
        for k in range(self._lib.l3es_kernel_kind_count()):
            ms, n, b = ctypes.c_double(), ctypes.c_int64(), ctypes.c_double()
            _check(self._lib.l3es_plan_kernel_stats(self._h, k, ctypes.byref(ms), ctypes.byref(n),
                                                    ctypes.byref(b)), "l3es_plan_kernel_stats")
            if n.value:
                out[self._lib.l3es_kernel_kind_name(k).decode()] = (n.value, ms.value, b.value)
        return out

    @property
    def workspace_bytes(self) -> int:
        return int(self._lib.l3es_plan_workspace_bytes(self._h))

    SCHEDULE_KEYS = ("x_bulk", "y_radix8", "line_pair", "band_bulk")

    @property
    def schedule(self) -> dict:
        """The plan's kernel schedule (l3es_plan_get_schedule) as {name: 0 or 1}; line_pair
        is 2 or 3 for the radix-16 line passes (N = 256; 3 fed by bulk copies); x_bulk
        selects the bulk-copy x passes in 3D and 2-column x-pass tiles in 2D."""
        v = (ctypes.c_int32 * 4)()
        _check(self._lib.l3es_plan_get_schedule(self._h, v), "l3es_plan_get_schedule")
        return dict(zip(self.SCHEDULE_KEYS, list(v)))

    def set_schedule(self, sched: dict) -> None:
        cur = self.schedule
        cur.update(sched)
        v = (ctypes.c_int32 * 4)(*[int(cur[k]) for k in self.SCHEDULE_KEYS])
        _check(self._lib.l3es_plan_set_schedule(self._h, v), "l3es_plan_set_schedule")

    STEP_FORMS = ("whole_spectrum", "closed_form_outside_rows", "band_fused")

    @property
    def step_form(self) -> int:
        """Form of the explicit RK4 step (l3es_plan_get_step_form): 0 one elementwise
        update of the whole spectrum per stage, 1 the closed form of the linear decay
        outside the dealiased rows, 2 the stage combination fused into the band pass
        (plans start at 2 in 3D, 1 in 2D). All forms compute the reference's RK4 step."""
        v = ctypes.c_int32()
        _check(self._lib.l3es_plan_get_step_form(self._h, ctypes.byref(v)), "l3es_plan_get_step_form")
        return int(v.value)

    @step_form.setter
    def step_form(self, form: int) -> None:
        _check(self._lib.l3es_plan_set_step_form(self._h, int(form)), "l3es_plan_set_step_form")

    def autotune(self, cache_path=None, stream=None) -> dict:
        """Pick the fastest kernel schedule for this plan (l3es_plan_autotune); cache_path
        defaults to $L3ES_TUNE_CACHE or ~/.cache/l3es_gb300/schedules.txt ("" = no
        cache). Returns the chosen schedule."""
        if cache_path is None:
            cache_path = os.environ.get("L3ES_TUNE_CACHE",
                                        os.path.join(os.path.expanduser("~"), ".cache", "l3es_gb300", "schedules.txt"))
        if cache_path:
            os.makedirs(os.path.dirname(os.path.abspath(cache_path)), exist_ok=True)
        path = cache_path.encode() if cache_path else None
        _check(self._lib.l3es_plan_autotune(self._h, path, _stream(stream)), "l3es_plan_autotune")
        return self.schedule

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.l3es_plan_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _prod(s):
    p = 1
    for v in s:
        p *= int(v)
    return p


BACKENDS = {"nufft": 0, "dft": 1}


class InterpPlan:
    """Owns an ``l3es_interp_plan``: coarse spectrum, NUFFT grid, particle bins."""

    def __init__(self, dim: int, ckp_n: int, n_fine: int = 0, width: int = 6, np_max: int = 0, batch: int = 1):
        """batch > 1: one plan for `batch` trajectories of a batched step plan
        (l3es_interp_plan_create_batch): set_spectrum takes their [batch][3][...] fine
        spectra, interp their [batch][np][dim] positions, NUFFT only."""
        lib = load()
        h = ctypes.c_void_p()
        _check(lib.l3es_interp_plan_create_batch(int(dim), int(n_fine), int(ckp_n), int(width), int(np_max),
                                                 int(batch), ctypes.byref(h)), "l3es_interp_plan_create_batch")
        self._h, self._lib = h, lib
        self.dim, self.c, self.n_fine, self.width, self.np_max = int(dim), int(ckp_n), int(n_fine), int(width), int(np_max)
        self.batch = int(batch)

    @property
    def coarse_shape(self):
        c = self.c
        return (3, c, c, c) if self.dim == 3 else (3, c, c, 1)

    @property
    def coarse_spec_shape(self):
        c = self.c
        return (3, c, c, c // 2 + 1) if self.dim == 3 else (3, c, c // 2 + 1)

    def set_spectrum(self, u_hat_fine, stream=None) -> None:
        import torch

        n = self.n_fine
        want = self.batch * 3 * n ** (self.dim - 1) * (n // 2 + 1)
        if n > 0 and (u_hat_fine.dtype != torch.complex64 or u_hat_fine.numel() != want
                      or not u_hat_fine.is_contiguous()):
            raise ValueError(f"u_hat_fine must be a contiguous complex64 tensor of {want} values "
                             f"({self.batch} x 3 fine half spectra of {n})")
        _check(self._lib.l3es_interp_set_spectrum(self._h, _ptr(u_hat_fine), _stream(stream)),
               "l3es_interp_set_spectrum")

    def set_field(self, u_coarse, stream=None) -> None:
        if u_coarse.numel() != _prod(self.coarse_shape):
            raise ValueError(f"expected float32 {self.coarse_shape}, got {tuple(u_coarse.shape)}")
        _check(self._lib.l3es_interp_set_field(self._h, _ptr(u_coarse), _stream(stream)), "l3es_interp_set_field")

    def coarse_field(self, out, stream=None) -> None:
        if out.numel() != _prod(self.coarse_shape):
            raise ValueError(f"expected float32 {self.coarse_shape}")
        _check(self._lib.l3es_interp_coarse_field(self._h, _ptr(out), _stream(stream)), "l3es_interp_coarse_field")

    def coarse_spectrum(self, out, stream=None) -> None:
        _check(self._lib.l3es_interp_coarse_spectrum(self._h, _ptr(out), _stream(stream)),
               "l3es_interp_coarse_spectrum")

    def interp(self, r, u_r, backend: str = "nufft", dt: float = 0.0, r_out=None, stream=None) -> None:
        import torch

        if r.dtype != torch.float64 or u_r.dtype != torch.float64:
            raise ValueError("positions and velocities are float64 (np, dim)")
        lead = (self.batch,) if self.batch > 1 else ()
        if (r.shape != u_r.shape or r.shape[-1] != self.dim or r.dim() != 2 + len(lead)
                or tuple(r.shape[:len(lead)]) != lead or not r.is_contiguous() or not u_r.is_contiguous()):
            raise ValueError(f"expected contiguous {lead + ('np', self.dim)} arrays")
        if r_out is not None and (r_out.shape != r.shape or r_out.dtype != torch.float64 or not r_out.is_contiguous()):
            raise ValueError("r_out must match r")
        _check(self._lib.l3es_interp(self._h, _ptr(r), int(r.shape[-2]), _ptr(u_r), BACKENDS[backend], float(dt),
                                     _ptr(r_out), _stream(stream)), "l3es_interp")

    def advect_rk4(self, r, u_r, dt: float, r_out, backend: str = "nufft", stream=None) -> None:
        """RK4 particle advection through the current coarse field held fixed over the
        step (extension; the reference's step is explicit Euler): u_r <- u(r),
        r_out <- r advanced by one RK4 step of dt."""
        import torch

        for a in (r, u_r, r_out):
            if a.dtype != torch.float64 or a.dim() != 2 or a.shape != r.shape or a.shape[-1] != self.dim:
                raise ValueError(f"positions and velocities are float64 (np, {self.dim})")
        _check(self._lib.l3es_interp_advect_rk4(self._h, _ptr(r), int(r.shape[0]), _ptr(u_r), BACKENDS[backend],
                                                float(dt), _ptr(r_out), _stream(stream)), "l3es_interp_advect_rk4")

    def interp_vjp(self, r, lam, grad_fine, backend: str = "nufft", stream=None) -> None:
        """grad_fine <- dL/du_hat_fine for the velocities of set_spectrum(u_hat_fine) +
        interp(r) at fixed positions r, given lam = dL/du_r (float64 (np, dim))."""
        import torch

        if r.dtype != torch.float64 or lam.dtype != torch.float64 or r.shape != lam.shape or r.shape[-1] != self.dim:
            raise ValueError(f"positions and cotangents are float64 (np, {self.dim})")
        n = self.n_fine
        want = 3 * n ** (self.dim - 1) * (n // 2 + 1)
        if grad_fine.dtype != torch.complex64 or grad_fine.numel() != want:
            raise ValueError(f"grad_fine must be a complex64 fine half spectrum of {want} values")
        _check(self._lib.l3es_interp_vjp(self._h, _ptr(r), int(r.shape[0]), _ptr(lam), BACKENDS[backend],
                                         _ptr(grad_fine), _stream(stream)), "l3es_interp_vjp")

    def coarse_mse(self, u_hat_fine, target, loss, grad=None, stream=None) -> None:
        """loss[0] = mean((spectral_filtering(irfftn(u_hat_fine), c) - target)^2) and,
        when grad is given, its gradient with respect to u_hat_fine. Replaces the
        plan's coarse spectrum."""
        import torch

        if target.dtype != torch.float32 or target.numel() != self.dim * self.c**self.dim:
            raise ValueError(f"target must be float32 ({self.dim}, c, ...) with c = {self.c}")
        if loss.dtype != torch.float64:
            raise ValueError("loss is a float64 device tensor")
        _check(self._lib.l3es_interp_coarse_mse(self._h, _ptr(u_hat_fine), _ptr(target), _ptr(loss), _ptr(grad),
                                                _stream(stream)), "l3es_interp_coarse_mse")

    def particles_to_grid(self, r, u_r, out, stream=None) -> None:
        """real(ifftn(sum_j u_r[j] exp(-i k.r_j))) on the c^dim grid into out (float32,
        (3, c, c, c) or (3, c, c))."""
        import torch

        if r.dtype != torch.float64 or u_r.dtype != torch.float64:
            raise ValueError("positions and velocities are float64 (np, dim)")
        _check(self._lib.l3es_interp_particles_to_grid(self._h, _ptr(r), _ptr(u_r), int(r.shape[0]), _ptr(out),
                                                       _stream(stream)), "l3es_interp_particles_to_grid")

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.l3es_interp_plan_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class SphPlan:
    """Owns an ``l3es_sph_plan``: cell list and per-particle scratch for n^dim particles
    in the periodic box [0, box)^dim."""

    def __init__(self, dim: int, n: int, box: float = 2 * 3.141592653589793, np_max: int = 0):
        lib = load()
        h = ctypes.c_void_p()
        np_max = int(np_max) or int(n) ** int(dim)
        _check(lib.l3es_sph_plan_create(int(dim), int(n), float(box), np_max, ctypes.byref(h)),
               "l3es_sph_plan_create")
        self._h, self._lib = h, lib
        self.dim, self.n, self.box, self.np_max = int(dim), int(n), float(box), np_max

    def _pos(self, *arrays):
        import torch

        for a in arrays:
            if a.dtype != torch.float64 or a.dim() != 2 or a.shape[1] != self.dim:
                raise ValueError(f"expected float64 (np, {self.dim}) arrays")
            if a.shape[0] != arrays[0].shape[0]:
                raise ValueError("particle arrays differ in length")
        return int(arrays[0].shape[0])

    def density(self, r, rho, stream=None) -> None:
        n = self._pos(r)
        if rho.numel() != n:
            raise ValueError("rho must hold one float64 per particle")
        _check(self._lib.l3es_sph_density(self._h, _ptr(r), n, _ptr(rho), _stream(stream)), "l3es_sph_density")

    def relax_acceleration(self, r, acc, u_ref: float, stream=None) -> None:
        n = self._pos(r, acc)
        _check(self._lib.l3es_sph_relax_acceleration(self._h, _ptr(r), n, float(u_ref), _ptr(acc), _stream(stream)),
               "l3es_sph_relax_acceleration")

    def forces(self, r, u, acc_p, acc_visc, acc_tvf, u_ref: float, stream=None) -> None:
        n = self._pos(r, u, acc_p, acc_visc, acc_tvf)
        _check(self._lib.l3es_sph_forces(self._h, _ptr(r), _ptr(u), n, float(u_ref), _ptr(acc_p), _ptr(acc_visc),
                                         _ptr(acc_tvf), _stream(stream)), "l3es_sph_forces")

    def relax_velocity(self, r0, u_r, u_out, dt: float, relax_dt_factor: float, u_ref: float, r_out=None,
                       stream=None) -> None:
        n = self._pos(r0, u_r, u_out) if r_out is None else self._pos(r0, u_r, u_out, r_out)
        _check(self._lib.l3es_sph_relax_velocity(self._h, _ptr(r0), _ptr(u_r), n, float(dt), float(relax_dt_factor),
                                                 float(u_ref), _ptr(u_out), _ptr(r_out), _stream(stream)),
               "l3es_sph_relax_velocity")

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.l3es_sph_plan_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def shift(r, dr, scale: float = 1.0, box: float = 2 * 3.141592653589793, out=None, stream=None):
    """shift_fn(r, scale * dr) on the GPU (float64 tensors); returns `out`."""
    import torch

    if out is None:
        out = torch.empty_like(r)
    _check(load().l3es_shift(_ptr(r), _ptr(dr), int(r.numel()), float(scale), float(box), _ptr(out),
                             _stream(stream)), "l3es_shift")
    return out


def interp_dft_noalloc(dim: int, n_fine: int, ckp_n: int, u_hat_fine, r, u_r, stream=None) -> None:
    """Exact spectral interpolation from a fine spectrum without any device
    allocation by the library (``l3es_interp_dft_noalloc``), for hosts that own all
    device memory themselves. The caller provides every input and output tensor;
    the library's fixed scratch limits ckp_n to 32 (3D) or 64 (2D)."""
    import torch

    dim, n_fine, ckp_n = int(dim), int(n_fine), int(ckp_n)
    if dim not in (2, 3):
        raise ValueError("dim must be 2 or 3")
    if r.dtype != torch.float64 or u_r.dtype != torch.float64 or r.shape != u_r.shape:
        raise ValueError("positions and velocities are float64 (np, dim)")
    if r.dim() != 2 or r.shape[1] != dim:
        raise ValueError(f"positions and velocities must be (np, {dim}) arrays, got {tuple(r.shape)}")
    if n_fine < 2 or n_fine & (n_fine - 1):
        raise ValueError("n_fine must be a power of two")
    want = 3 * n_fine ** (dim - 1) * (n_fine // 2 + 1)
    if u_hat_fine.dtype != torch.complex64 or u_hat_fine.numel() != want or not u_hat_fine.is_contiguous():
        raise ValueError(f"u_hat_fine must be a contiguous complex64 half spectrum of {want} values "
                         f"(3, {n_fine}{', ' + str(n_fine) if dim == 3 else ''}, {n_fine // 2 + 1}), "
                         f"got {u_hat_fine.dtype} {tuple(u_hat_fine.shape)}")
    if not (r.is_contiguous() and u_r.is_contiguous()):
        raise ValueError("positions and velocities must be contiguous")
    _check(load().l3es_interp_dft_noalloc(int(dim), int(n_fine), int(ckp_n), _ptr(u_hat_fine), _ptr(r),
                                          int(r.shape[0]), _ptr(u_r), _stream(stream)), "l3es_interp_dft_noalloc")


class _CaptureStream:
    """A capturing stream handle, accepted wherever a ``stream=`` argument is."""

    def __init__(self, handle: int):
        self.cuda_stream = handle


class Graph:
    """Library calls recorded once and replayed as one CUDA graph launch.

        cap = Graph.begin()
        plan_a.step(uh_a, 1, stream=cap); plan_b.step(uh_b, 1, stream=cap)
        g = Graph.end(cap)
        for _ in range(steps): g.launch()
    """

    def __init__(self, handle):
        self._h = handle
        self._lib = load()

    @staticmethod
    def begin() -> _CaptureStream:
        h = ctypes.c_void_p()
        _check(load().l3es_graph_begin(ctypes.byref(h)), "l3es_graph_begin")
        return _CaptureStream(h.value)

    @staticmethod
    def fork(cap: _CaptureStream) -> _CaptureStream:
        """A branch of the recording: calls given it run concurrently with the rest of
        the recording until join(cap, branch)."""
        h = ctypes.c_void_p()
        _check(load().l3es_graph_fork(cap.cuda_stream, ctypes.byref(h)), "l3es_graph_fork")
        return _CaptureStream(h.value)

    @staticmethod
    def join(cap: _CaptureStream, branch: _CaptureStream) -> None:
        _check(load().l3es_graph_join(cap.cuda_stream, branch.cuda_stream), "l3es_graph_join")

    @staticmethod
    def end(cap: _CaptureStream) -> "Graph":
        h = ctypes.c_void_p()
        _check(load().l3es_graph_end(cap.cuda_stream, ctypes.byref(h)), "l3es_graph_end")
        return Graph(h)

    def launch(self, stream=None) -> None:
        _check(self._lib.l3es_graph_launch(self._h, _stream(stream)), "l3es_graph_launch")

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.l3es_graph_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
