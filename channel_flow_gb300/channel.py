"""ctypes binding of include/chflow.h and the Channel class.

Status codes and error strings come straight from the library; a non-zero
status raises ChannelError carrying chf_last_error().
"""
import ctypes
import os

import numpy as np

from .config import ChannelConfig
from .fields import FIELD_NAMES, MEAN_NAMES

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libchflow.so")

PRECISION = {"fp64": 0, "mixed": 1, "mixed_fp64solve": 2}
STATUS = {0: "CHF_OK", -1: "CHF_E_INVALID", -2: "CHF_E_CUDA", -3: "CHF_E_NOMEM",
          -4: "CHF_E_STATE", -5: "CHF_E_NUMERIC"}

# Every entry point declared in include/chflow.h.
EXPORTS = ("chf_create", "chf_destroy", "chf_last_error", "chf_upload_state",
           "chf_download_state", "chf_getnonlinear", "chf_solve", "chf_step", "chf_step_host",
           "chf_synchronize", "chf_diagnostics", "chf_kernels_per_step", "chf_device_field",
           "chf_set_stream", "chf_profile_enable", "chf_profile_reset", "chf_profile_read",
           "chf_diagnostics_static", "chf_write_restart", "chf_read_restart",
           "chf_batch_create", "chf_batch_destroy", "chf_batch_last_error", "chf_batch_size",
           "chf_batch_handle", "chf_batch_step", "chf_batch_synchronize",
           "chf_set_flow_rate", "chf_get_flow_rate", "chf_statistics", "chf_pressure",
           "chf_transform", "chf_cfl", "chf_physical_velocity", "chf_write_velocity",
           "chf_autotune", "chf_tuning", "chf_set_launch_shape", "chf_test_wait_timeout")


class ChannelError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{STATUS.get(code, code)}: {msg}")
        self.code = code


class CConfig(ctypes.Structure):
    _fields_ = [("nnx", ctypes.c_int), ("nny", ctypes.c_int), ("nnz", ctypes.c_int),
                ("aphi", ctypes.c_double), ("beta", ctypes.c_double), ("dt", ctypes.c_double),
                ("re", ctypes.c_double), ("re_p", ctypes.c_double), ("precision", ctypes.c_int),
                ("zpad", ctypes.c_int), ("device", ctypes.c_int)]


class CStats(ctypes.Structure):
    _fields_ = [(n, ctypes.c_double) for n in ("u_tau_top", "u_tau_bottom", "re_tau_top", "re_tau_bottom",
                                               "re_centre", "re_bulk", "bulk_velocity", "energy")]


class CDiag(ctypes.Structure):
    _fields_ = [("energy", ctypes.c_double), ("wall_shear_top", ctypes.c_double),
                ("wall_shear_bottom", ctypes.c_double), ("max_abs", ctypes.c_double),
                ("finite", ctypes.c_int)]


_lib = None


def load_library(path: str = None):
    """Load libchflow.so (build it with channel_flow_gb300.build.build())."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise ChannelError(-2, f"CUDA library not found at {p}; run channel_flow_gb300.build.build()")
    L = ctypes.CDLL(p)
    dp = ctypes.POINTER(ctypes.c_double)
    vp = ctypes.c_void_p
    L.chf_create.argtypes = [ctypes.POINTER(CConfig), ctypes.POINTER(vp)]
    L.chf_destroy.argtypes = [vp]
    L.chf_last_error.argtypes = [vp]
    L.chf_last_error.restype = ctypes.c_char_p
    L.chf_upload_state.argtypes = [vp] + [dp] * 14
    L.chf_download_state.argtypes = [vp] + [dp] * 14
    for name in ("chf_getnonlinear", "chf_solve", "chf_synchronize"):
        getattr(L, name).argtypes = [vp]
    L.chf_step.argtypes = [vp, ctypes.c_int]
    L.chf_step_host.argtypes = [vp, ctypes.c_int] + [dp] * 14
    L.chf_diagnostics.argtypes = [vp, ctypes.POINTER(CDiag)]
    L.chf_kernels_per_step.argtypes = [vp]
    L.chf_device_field.argtypes = [vp, ctypes.c_int, ctypes.POINTER(vp)]
    L.chf_set_stream.argtypes = [vp, vp]
    L.chf_profile_enable.argtypes = [vp, ctypes.c_int]
    L.chf_profile_reset.argtypes = [vp]
    L.chf_profile_read.argtypes = [vp, ctypes.c_int, ctypes.POINTER(ctypes.c_char_p),
                                   ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_double)]
    L.chf_diagnostics_static.argtypes = [ctypes.c_int] * 3 + [vp] * 6 + [dp, ctypes.POINTER(CDiag), vp]
    for name in ("chf_write_restart", "chf_read_restart"):
        getattr(L, name).argtypes = [vp, ctypes.c_char_p, ctypes.c_int, ctypes.c_int, ctypes.c_int]
    L.chf_batch_create.argtypes = [ctypes.c_int, ctypes.POINTER(CConfig), ctypes.POINTER(vp)]
    L.chf_batch_last_error.argtypes = [vp]
    L.chf_batch_last_error.restype = ctypes.c_char_p
    for name in ("chf_batch_destroy", "chf_batch_size", "chf_batch_synchronize"):
        getattr(L, name).argtypes = [vp]
    L.chf_batch_handle.argtypes = [vp, ctypes.c_int, ctypes.POINTER(vp)]
    L.chf_batch_step.argtypes = [vp, ctypes.c_int]
    L.chf_set_flow_rate.argtypes = [vp, ctypes.c_double]
    L.chf_get_flow_rate.argtypes = [vp, dp, dp, dp]
    L.chf_statistics.argtypes = [vp, dp, ctypes.POINTER(CStats)]
    L.chf_pressure.argtypes = [vp, dp]
    L.chf_transform.argtypes = [vp, ctypes.c_int, dp]
    L.chf_autotune.argtypes = [vp, ctypes.c_int]
    L.chf_test_wait_timeout.argtypes = [vp, ctypes.c_int]
    L.chf_tuning.argtypes = [vp, ctypes.c_char_p, ctypes.c_int]
    L.chf_set_launch_shape.argtypes = [vp, ctypes.c_char_p, ctypes.c_int]
    L.chf_cfl.argtypes = [vp, dp, dp, dp]
    L.chf_physical_velocity.argtypes = [vp, dp, dp]
    L.chf_write_velocity.argtypes = [vp, ctypes.c_char_p, ctypes.c_int, ctypes.c_int, dp]
    for name in EXPORTS:
        getattr(L, name).restype = getattr(L, name).restype or ctypes.c_int
    L.chf_last_error.restype = ctypes.c_char_p
    L.chf_batch_last_error.restype = ctypes.c_char_p
    if path is None:
        _lib = L
    return L


def _dptr(a):
    if a is None:
        return None
    assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def make_cconfig(cfg: ChannelConfig, precision="fp64", zpad=0, device=0) -> CConfig:
    return CConfig(cfg.nnx, cfg.nny, cfg.nnz, cfg.aphi, cfg.beta, cfg.dt, cfg.re, cfg.re_p,
                   PRECISION[precision] if isinstance(precision, str) else int(precision),
                   int(zpad), int(device))


class Channel:
    """One channel resident on one GPU (a chf_handle)."""

    def __init__(self, cfg: ChannelConfig, precision="fp64", zpad=0, device=0):
        self.L = load_library()
        self.cfg = cfg
        self.shape = (cfg.nnz + 1, cfg.nny, cfg.nnx)
        self.h = ctypes.c_void_p()
        c = make_cconfig(cfg, precision, zpad, device)
        rc = self.L.chf_create(ctypes.byref(c), ctypes.byref(self.h))
        if rc != 0:
            raise ChannelError(rc, self.L.chf_last_error(None).decode())

    def _check(self, rc):
        if rc != 0:
            raise ChannelError(rc, self.L.chf_last_error(self.h).decode())

    def close(self):
        if getattr(self, "h", None) and self.h.value:
            self.L.chf_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def upload_state(self, st: dict):
        arrs = []
        for k in FIELD_NAMES:
            a = st.get(k)
            if a is not None:
                a = np.ascontiguousarray(a, dtype=np.float64)
                if a.shape != self.shape:
                    raise ChannelError(-1, f"{k}: shape {a.shape} != {self.shape}")
            arrs.append(a)
        for k in MEAN_NAMES:
            a = st.get(k)
            if a is not None:
                a = np.ascontiguousarray(a, dtype=np.float64)
                if a.shape != (self.cfg.nnz + 1, 2):
                    raise ChannelError(-1, f"{k}: shape {a.shape} != {(self.cfg.nnz + 1, 2)}")
            arrs.append(a)
        self._check(self.L.chf_upload_state(self.h, *[_dptr(a) for a in arrs]))

    def download_state(self, out: dict = None) -> dict:
        """Copy the module arrays device -> host, into ``out`` (C-contiguous
        float64 arrays, e.g. pinned buffers) when given."""
        if out is None:
            out = {k: np.empty(self.shape) for k in FIELD_NAMES}
            out.update({k: np.empty((self.cfg.nnz + 1, 2)) for k in MEAN_NAMES})
        self._check(self.L.chf_download_state(
            self.h, *[_dptr(out[k]) for k in FIELD_NAMES], *[_dptr(out[k]) for k in MEAN_NAMES]))
        return out

    def step_host(self, st: dict, n: int = 1) -> dict:
        """Advance the host module arrays in ``st`` by ``n`` steps in place
        (chf_step_host: upload, steps and download overlapped; page-locked
        arrays give the full link bandwidth).  Every array is required,
        C-contiguous float64 and writable."""
        arrs = []
        for k, shape in [(k, self.shape) for k in FIELD_NAMES] + [(k, (self.cfg.nnz + 1, 2)) for k in MEAN_NAMES]:
            a = st.get(k)
            if a is None or a.dtype != np.float64 or not a.flags.c_contiguous or not a.flags.writeable:
                raise ChannelError(-1, f"{k}: a writable C-contiguous float64 array is required")
            if a.shape != shape:
                raise ChannelError(-1, f"{k}: shape {a.shape} != {shape}")
            arrs.append(a)
        self._check(self.L.chf_step_host(self.h, int(n), *[_dptr(a) for a in arrs]))
        return st

    def getnonlinear(self):
        self._check(self.L.chf_getnonlinear(self.h))

    def solve(self):
        self._check(self.L.chf_solve(self.h))

    def step(self, n=1):
        self._check(self.L.chf_step(self.h, int(n)))

    def synchronize(self):
        self._check(self.L.chf_synchronize(self.h))

    def diagnostics(self) -> dict:
        d = CDiag()
        rc = self.L.chf_diagnostics(self.h, ctypes.byref(d))
        if rc not in (0, -5):
            self._check(rc)
        return {"energy": d.energy, "wall_shear_top": d.wall_shear_top,
                "wall_shear_bottom": d.wall_shear_bottom, "max_abs": d.max_abs,
                "finite": bool(d.finite)}

    def write_restart(self, directory: str, nproc: int = 1, tag: int = 2, istep: int = -1):
        """The reference's per-rank restart files (output, poiseuilleflow.f90:2460-2504)
        from the device state; call after getnonlinear, as the reference does."""
        self._check(self.L.chf_write_restart(self.h, os.fsencode(directory), int(nproc), int(tag), int(istep)))

    def read_restart(self, directory: str, nproc: int = 1, tag: int = 2, istep: int = -1):
        """Load the reference's per-rank restart files (initial,
        poiseuilleflow.f90:1873-1917) into the device state; continue with solve()."""
        self._check(self.L.chf_read_restart(self.h, os.fsencode(directory), int(nproc), int(tag), int(istep)))

    def statistics(self) -> dict:
        """Plane statistics at the Gauss-Lobatto points and the scalar
        diagnostics of the reference's statistics routine."""
        prof = np.zeros((10, self.cfg.nnz + 1))
        st = CStats()
        self._check(self.L.chf_statistics(self.h, _dptr(prof), ctypes.byref(st)))
        out = {n: getattr(st, n) for n, _ in CStats._fields_}
        for i, n in enumerate(("z", "u", "v", "w", "uu", "vv", "ww", "uv", "uw", "vw")):
            out[n] = prof[i]
        return out

    def pressure(self) -> np.ndarray:
        """Total-head pressure P = p + |u|^2/2 of the current state (after a
        solve), Chebyshev coefficients in the field layout."""
        out = np.zeros(self.shape)
        self._check(self.L.chf_pressure(self.h, _dptr(out)))
        return out

    def test_wait_timeout(self, wait_us: int):
        """Arm the test of the tensor-core pipeline's bounded waits: the next
        GEMM launch leaves its first stage empty, its waits run out after
        wait_us and the next synchronize reports CHF_E_CUDA."""
        self._check(self.L.chf_test_wait_timeout(self.h, int(wait_us)))

    def autotune(self, reps: int = 3) -> str:
        """Pick launch shapes and FFT radix orders by timing steps of the
        current state (chf_autotune); returns the choice as text."""
        self._check(self.L.chf_autotune(self.h, int(reps)))
        return self.tuning()

    def tuning(self) -> str:
        buf = ctypes.create_string_buffer(1024)
        self._check(self.L.chf_tuning(self.h, buf, len(buf)))
        return buf.value.decode()

    def set_launch_shape(self, name: str, value: int) -> None:
        """One launch shape by name (chf_set_launch_shape): "inc_modes",
        "inc_columns", "inc_rows", "kxb", "xr", "zl_c2v" or "zl_curl"."""
        self._check(self.L.chf_set_launch_shape(self.h, name.encode(), int(value)))

    def transform(self, isign: int, u: np.ndarray) -> np.ndarray:
        """transform (poiseuilleflow.f90:919-1005) of one array in the field
        layout on the device: isign = 1 spectral -> physical grid, -1 back.
        Returns a new array."""
        a = np.ascontiguousarray(u, dtype=np.float64).copy()
        if a.shape != self.shape:
            raise ChannelError(-1, f"shape {a.shape} != {self.shape}")
        self._check(self.L.chf_transform(self.h, int(isign), _dptr(a)))
        return a

    def cfl(self) -> dict:
        """CFL_X (streamwise), CFL_Y (wall-normal), CFL_Z (spanwise) of the
        current state, as statistics prints them."""
        x, y, z = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        self._check(self.L.chf_cfl(self.h, ctypes.byref(x), ctypes.byref(y), ctypes.byref(z)))
        return {"cfl_x": x.value, "cfl_y": y.value, "cfl_z": z.value}

    def physical_velocity(self, u0=None) -> np.ndarray:
        """(u + u0, w, v) on the physical grid, shape (3, nz+1, nny, nnx):
        the reference's ftmp(i, j, k, m) of the 3Ddata dump."""
        out = np.empty((3,) + self.shape)
        p0 = None if u0 is None else np.ascontiguousarray(u0, dtype=np.float64)
        self._check(self.L.chf_physical_velocity(self.h, _dptr(p0), _dptr(out)))
        return out

    def write_velocity(self, directory: str, nproc: int = 1, istep: int = 0, u0=None):
        """The 3Ddata dump files velocity<istep>.<rank>.dat in directory."""
        p0 = None if u0 is None else np.ascontiguousarray(u0, dtype=np.float64)
        self._check(self.L.chf_write_velocity(self.h, os.fsencode(directory), int(nproc), int(istep), _dptr(p0)))

    def set_flow_rate(self, bulk_velocity: float):
        """Hold the bulk velocity at bulk_velocity (> 0) by adjusting the mean
        pressure gradient every step; 0 switches the control off."""
        self._check(self.L.chf_set_flow_rate(self.h, float(bulk_velocity)))

    def flow_rate(self) -> dict:
        t, u, p = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        self._check(self.L.chf_get_flow_rate(self.h, ctypes.byref(t), ctypes.byref(u), ctypes.byref(p)))
        return {"target": t.value, "bulk_velocity": u.value, "dpdx_correction": p.value}

    def kernels_per_step(self) -> int:
        return int(self.L.chf_kernels_per_step(self.h))

    def set_stream(self, stream_ptr):
        """Run on a caller CUDA stream (an integer cudaStream_t, e.g.
        torch.cuda.Stream().cuda_stream); None restores the own stream."""
        self._check(self.L.chf_set_stream(self.h, ctypes.c_void_p(stream_ptr or 0)))

    def profile(self, on=True):
        self._check(self.L.chf_profile_enable(self.h, int(bool(on))))

    def profile_reset(self):
        self._check(self.L.chf_profile_reset(self.h))

    def profile_report(self) -> dict:
        """{kernel name: (launches, total device ms)} since the last reset."""
        out = {}
        i = 0
        while True:
            name = ctypes.c_char_p()
            n = ctypes.c_int()
            ms = ctypes.c_double()
            rc = self.L.chf_profile_read(self.h, i, ctypes.byref(name), ctypes.byref(n), ctypes.byref(ms))
            if rc != 0:
                break
            out[name.value.decode()] = (n.value, ms.value)
            i += 1
        return out


class _Borrowed(Channel):
    """A channel owned by a Batch: every Channel call, no destroy."""

    def __init__(self, L, h, cfg):
        self.L = L
        self.cfg = cfg
        self.shape = (cfg.nnz + 1, cfg.nny, cfg.nnx)
        self.h = h

    def close(self):
        self.h = ctypes.c_void_p()


class Batch:
    """An ensemble of independent channels on one GPU (a chf_batch)."""

    def __init__(self, cfgs, precision="fp64", zpad=0, device=0):
        self.L = load_library()
        cfgs = list(cfgs)
        precs = precision if isinstance(precision, (list, tuple)) else [precision] * len(cfgs)
        zpads = zpad if isinstance(zpad, (list, tuple)) else [zpad] * len(cfgs)
        arr = (CConfig * len(cfgs))(*[make_cconfig(c, p, z, device) for c, p, z in zip(cfgs, precs, zpads)])
        self.b = ctypes.c_void_p()
        rc = self.L.chf_batch_create(len(cfgs), arr, ctypes.byref(self.b))
        if rc != 0:
            raise ChannelError(rc, self.L.chf_batch_last_error(None).decode())
        self.channels = []
        for i, c in enumerate(cfgs):
            h = ctypes.c_void_p()
            self._check(self.L.chf_batch_handle(self.b, i, ctypes.byref(h)))
            self.channels.append(_Borrowed(self.L, h, c))

    def _check(self, rc):
        if rc != 0:
            raise ChannelError(rc, self.L.chf_batch_last_error(self.b).decode())

    def __len__(self):
        return len(self.channels)

    def __getitem__(self, i) -> Channel:
        return self.channels[i]

    def step(self, n=1):
        self._check(self.L.chf_batch_step(self.b, int(n)))

    def synchronize(self):
        self._check(self.L.chf_batch_synchronize(self.b))

    def close(self):
        if getattr(self, "b", None) and self.b.value:
            for c in self.channels:
                c.close()
            self.L.chf_batch_destroy(self.b)
            self.b = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()
