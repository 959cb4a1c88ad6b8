"""ctypes view of the CPU oracle (test infrastructure only).

Imported by tests/, __graft_entry__.smoke() and the CPU-baseline leg of
bench.py to CHECK or TIME against; the product package never imports it.
"""
import ctypes
import os

import numpy as np

from .build_oracle import build

FIELDS = ["vnp1", "omegaynp1", "unp1", "wnp1", "omegaxnp1", "omegaznp1", "rhsvn", "rhsomegayn"]
MEANS = ["clamb1n", "clamb1nm1", "clamb3n", "clamb3nm1", "au0", "w0"]

_lib = None


def lib():
    global _lib
    if _lib is None:
        path = build()
        L = ctypes.CDLL(path)
        dp = ctypes.POINTER(ctypes.c_double)
        L.orc_create.restype = ctypes.c_void_p
        L.orc_create.argtypes = [ctypes.c_int] * 3 + [ctypes.c_double] * 5
        L.orc_destroy.argtypes = [ctypes.c_void_p]
        L.orc_field.restype = dp
        L.orc_field.argtypes = [ctypes.c_void_p, ctypes.c_int]
        L.orc_mean.restype = dp
        L.orc_mean.argtypes = [ctypes.c_void_p, ctypes.c_int]
        for name in ("orc_setup", "orc_getnonlinear", "orc_solve", "orc_velocity_all"):
            getattr(L, name).argtypes = [ctypes.c_void_p]
        L.orc_step.argtypes = [ctypes.c_void_p, ctypes.c_int]
        L.orc_transform.argtypes = [ctypes.c_void_p, ctypes.c_int, dp]
        L.orc_fft.argtypes = [ctypes.c_int, ctypes.c_int, dp]
        L.orc_dz.argtypes = [dp, ctypes.c_int]
        L.orc_getlamb.argtypes = [ctypes.c_void_p, dp, dp, dp, ctypes.c_int]
        L.orc_matrices.argtypes = [ctypes.c_void_p, ctypes.c_double, dp, dp, dp, dp]
        L.orc_scheb.argtypes = [ctypes.c_void_p, dp, dp, dp, dp]
        L.orc_set_threads.argtypes = [ctypes.c_int]
        _lib = L
    return _lib


def _ptr(a):
    assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def set_threads(n: int) -> None:
    lib().orc_set_threads(int(n))


class Oracle:
    """One channel on the CPU, state held in the reference's Fortran layout.

    Arrays are exposed as NumPy views of shape (nz+1, ny+1, nx+1) (C order),
    i.e. the Fortran (0:nx,0:ny,0:nz) array with x fastest.
    """

    def __init__(self, nnx, nny, nnz, aphi, beta, dt, re, re_p):
        self.L = lib()
        self.shape = (nnz + 1, nny, nnx)
        self.nz = nnz
        self.h = self.L.orc_create(nnx, nny, nnz, aphi, beta, dt, re, re_p)

    @classmethod
    def from_config(cls, cfg):
        return cls(cfg.nnx, cfg.nny, cfg.nnz, cfg.aphi, cfg.beta, cfg.dt, cfg.re, cfg.re_p)

    def __del__(self):
        if getattr(self, "h", None):
            self.L.orc_destroy(self.h)
            self.h = None

    def field(self, name):
        p = self.L.orc_field(self.h, FIELDS.index(name))
        n = self.shape[0] * self.shape[1] * self.shape[2]
        return np.ctypeslib.as_array(p, shape=(n,)).reshape(self.shape)

    def mean(self, name):
        p = self.L.orc_mean(self.h, MEANS.index(name))
        return np.ctypeslib.as_array(p, shape=(2 * (self.nz + 1),)).reshape(self.nz + 1, 2)

    def set_state(self, state):
        for k in FIELDS:
            if k in state:
                self.field(k)[...] = state[k]
        for k in MEANS:
            if k in state:
                self.mean(k)[...] = state[k]

    def get_state(self):
        s = {k: self.field(k).copy() for k in FIELDS}
        s.update({k: self.mean(k).copy() for k in MEANS})
        return s

    def setup(self):
        self.L.orc_setup(self.h)

    def getnonlinear(self):
        self.L.orc_getnonlinear(self.h)

    def solve(self):
        self.L.orc_solve(self.h)

    def step(self, n=1):
        self.L.orc_step(self.h, int(n))

    def velocity_all(self):
        self.L.orc_velocity_all(self.h)

    def transform(self, isign, u):
        u = np.ascontiguousarray(u, dtype=np.float64).copy()
        self.L.orc_transform(self.h, int(isign), _ptr(u))
        return u

    def getlamb(self, u, omega, with_rep=False):
        out = np.zeros(self.shape)
        self.L.orc_getlamb(self.h, _ptr(np.ascontiguousarray(u)), _ptr(np.ascontiguousarray(omega)),
                           _ptr(out), int(with_rep))
        return out

    def matrices(self, kmn):
        Z = self.nz + 1
        av, ae, xv, xe = (np.zeros((Z, Z)) for _ in range(4))
        self.L.orc_matrices(self.h, float(kmn), _ptr(av), _ptr(ae), _ptr(xv), _ptr(xe))
        # stored column-major: transpose to row-major views
        return av.T.copy(), ae.T.copy(), xv.T.copy(), xe.T.copy()

    def scheb(self):
        Z = self.nz + 1
        t = [np.zeros((Z, Z)) for _ in range(4)]
        self.L.orc_scheb(self.h, *[_ptr(a) for a in t])
        return [a.T.copy() for a in t]


def fft(x, sign):
    """Unnormalised complex DFT with the FFTW sign convention."""
    a = np.ascontiguousarray(np.asarray(x, dtype=np.complex128)).copy()
    v = a.view(np.float64)
    lib().orc_fft(len(a), int(sign), _ptr(v))
    return a


def dz(v):
    a = np.ascontiguousarray(np.asarray(v, dtype=np.float64)).copy()
    lib().orc_dz(_ptr(a), len(a) - 1)
    return a
