"""ctypes binding of the dugks_gb300 C ABI (include/dugks_gb300.h).

The Python-facing mirror of the reference's solver interface
(Kairzhan/DUGKS-GPU src/dugks.h:1-9, src/output.h:1-5): an `Engine` owns one
`dg_t` handle.  Every call goes through libdugks_gb300.so; there is no Python
or CPU implementation of the step behind it, and importing this module fails
loudly when the library has not been built.

Host arrays are numpy float64:
  state (dump order):  shape (nz, ny, nx, 19)   -- ddf%08d.dat element order
  ghosted macro:       shape (nz+2, ny+2, nx+2)
"""
import ctypes
import os

import numpy as np

# workload and config.txt builders (pure Python, no library): re-exported here
from workloads import (REFERENCE_KEYS, channel_config, laminar_config, make_config,  # noqa: F401
                       taylor_green_config, tanh_alpha_for_first_face)

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libdugks_gb300.so")

DG_OK = 0
DG_ERR_CONFIG = -1
DG_ERR_IO = -2
DG_ERR_SHAPE = -3
DG_ERR_CUDA = -4
DG_ERR_NUMERIC = -5
DG_ERR_ARG = -6
DG_ERR_UNSUPPORTED = -7

PREC = {"fp64": 0, "fp32": 1, "fp16": 2, "bf16": 3}

DG_BUF_F = 0   # f-tilde, SoA
DG_BUF_FB = 1  # f-bar-plus, SoA with x ghost columns


class DugksError(RuntimeError):
    def __init__(self, code, message):
        super().__init__(f"dugks_gb300 status {code}: {message}")
        self.code = code


class Info(ctypes.Structure):
    _fields_ = [("nx", ctypes.c_int), ("ny", ctypes.c_int), ("nz", ctypes.c_int), ("pitch", ctypes.c_int),
                ("pop_stride", ctypes.c_longlong), ("precision", ctypes.c_int),
                ("periodic", ctypes.c_int * 3), ("mesh", ctypes.c_int), ("recon", ctypes.c_int),
                ("perturb", ctypes.c_int), ("istep0", ctypes.c_int), ("nsteps", ctypes.c_int),
                ("noutput2", ctypes.c_int), ("ndump", ctypes.c_int), ("restart", ctypes.c_int),
                ("nrestart", ctypes.c_int), ("dx", ctypes.c_double), ("dy", ctypes.c_double),
                ("dz", ctypes.c_double), ("dt", ctypes.c_double), ("visc", ctypes.c_double),
                ("tau", ctypes.c_double), ("xwidth", ctypes.c_double), ("ywidth", ctypes.c_double),
                ("zwidth", ctypes.c_double), ("ambient", ctypes.c_double * 3), ("bw0", ctypes.c_double),
                ("bw1", ctypes.c_double), ("bw2", ctypes.c_double), ("fw0", ctypes.c_double),
                ("fw1", ctypes.c_double), ("fw2", ctypes.c_double), ("hbm_bytes_per_cell", ctypes.c_double)]


_lib = None
_D = ctypes.POINTER(ctypes.c_double)


def lib():
    """Load libdugks_gb300.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"{LIB_PATH} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'`")
    L = ctypes.CDLL(LIB_PATH)
    H = ctypes.c_void_p
    sig = {
        "dg_create": (ctypes.c_int, [ctypes.c_char_p, ctypes.POINTER(H)]),
        "dg_create_from_text": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_char_p, ctypes.POINTER(H)]),
        "dg_destroy": (ctypes.c_int, [H]),
        "dg_last_error": (ctypes.c_char_p, [H]),
        "dg_get_info": (ctypes.c_int, [H, ctypes.POINTER(Info)]),
        "dg_set_stream": (ctypes.c_int, [H, ctypes.c_void_p]),
        "dg_step": (ctypes.c_int, [H, ctypes.c_int]),
        "dg_run": (ctypes.c_int, [H, ctypes.c_int, ctypes.c_int]),
        "dg_run_profiled": (ctypes.c_int, [H, ctypes.c_int, ctypes.c_int, _D]),
        "dg_run_between": (ctypes.c_int, [H, ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]),
        "dg_sync": (ctypes.c_int, [H]),
        "dg_selftest_wait_timeout": (ctypes.c_int, [H, ctypes.c_int, ctypes.POINTER(ctypes.c_longlong)]),
        "dg_upload_macro": (ctypes.c_int, [H]),
        "dg_copy_vel": (ctypes.c_int, [H, _D, _D, _D, _D]),
        "dg_stats_values": (ctypes.c_int, [H, _D, _D]),
        "dg_stats": (ctypes.c_int, [H, ctypes.c_int]),
        "dg_output_2d": (ctypes.c_int, [H, ctypes.c_int]),
        "dg_copy_ddf": (ctypes.c_int, [H, _D]),
        "dg_get_state": (ctypes.c_int, [H, _D]),
        "dg_set_state": (ctypes.c_int, [H, _D]),
        "dg_dump": (ctypes.c_int, [H, ctypes.c_int]),
        "dg_read_dump": (ctypes.c_int, [H, ctypes.c_int]),
        "dg_device_ptr": (ctypes.c_void_p, [H, ctypes.c_int]),
        "dg_moments": (ctypes.c_int, [H, _D]),
        "dg_get_mesh": (ctypes.c_int, [H, _D, _D]),
        "dg_stats_accumulate": (ctypes.c_int, [H]),
        "dg_stats_accumulated": (ctypes.c_int, [H, _D, ctypes.POINTER(ctypes.c_longlong)]),
        "dg_stats_reset": (ctypes.c_int, [H]),
        "dg_stats_values_noalloc": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                                    ctypes.c_int, ctypes.c_longlong, ctypes.c_double,
                                                    ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                                    ctypes.c_void_p, ctypes.c_void_p]),
        "dg_noalloc_last_error": (ctypes.c_char_p, []),
        "dg_spectral_stats": (ctypes.c_int, [H, _D, _D, ctypes.c_int]),
        "dg_output_spectral": (ctypes.c_int, [H, ctypes.c_int]),
        "dg_get_state_device": (ctypes.c_int, [H, ctypes.c_void_p]),
        "dg_set_state_device": (ctypes.c_int, [H, ctypes.c_void_p]),
        "dg_adjoint_step": (ctypes.c_int, [H, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
        "dg_run_store": (ctypes.c_int, [H, ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_longlong]),
        "dg_adjoint_run": (ctypes.c_int, [H, ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_longlong,
                                          ctypes.c_void_p]),
        "dg_set_force_field": (ctypes.c_int, [H, ctypes.c_int, _D]),
        "dg_field_grad": (ctypes.c_int, [H, _D, ctypes.c_int]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def _ptr(a):
    if a is None:
        return None
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(_D)


def last_error(h=None):
    return lib().dg_last_error(h).decode(errors="replace")


class Engine:
    """One dg_t handle.  `config` is config.txt text; files go to `workdir`."""

    def __init__(self, config=None, workdir=".", config_path=None):
        L = lib()
        h = ctypes.c_void_p()
        if config_path is not None:
            rc = L.dg_create(config_path.encode(), ctypes.byref(h))
        else:
            rc = L.dg_create_from_text(config.encode(), workdir.encode(), ctypes.byref(h))
        if rc != DG_OK:
            raise DugksError(rc, last_error(None))
        self._h = h
        self.info = Info()
        self._check(L.dg_get_info(self._h, ctypes.byref(self.info)))
        self.nx, self.ny, self.nz = self.info.nx, self.info.ny, self.info.nz

    def _check(self, rc):
        if rc != DG_OK:
            raise DugksError(rc, last_error(self._h))
        return rc

    def close(self):
        if getattr(self, "_h", None):
            lib().dg_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # stepping
    def step(self, istep):
        self._check(lib().dg_step(self._h, istep))

    def run(self, istep0, nsteps):
        self._check(lib().dg_run(self._h, istep0, nsteps))

    def run_between(self, istep0, nsteps, src_ptr=None, dst_ptr=None):
        """nsteps steps from the device state at src_ptr into dst_ptr (None: the engine's own state)."""
        self._check(lib().dg_run_between(self._h, istep0, nsteps, None if src_ptr is None else ctypes.c_void_p(src_ptr),
                                         None if dst_ptr is None else ctypes.c_void_p(dst_ptr)))

    def run_profiled(self, istep0, nsteps):
        """Run with per-kernel CUDA events; returns (ms of stage (a), ms of flux) summed over the steps."""
        ms = np.zeros(2)
        self._check(lib().dg_run_profiled(self._h, istep0, nsteps, _ptr(ms)))
        return float(ms[0]), float(ms[1])

    def sync(self):
        self._check(lib().dg_sync(self._h))

    def set_stream(self, stream_handle):
        self._check(lib().dg_set_stream(self._h, ctypes.c_void_p(stream_handle)))

    # state
    def get_state(self):
        a = np.empty((self.nz, self.ny, self.nx, 19), dtype=np.float64)
        self._check(lib().dg_get_state(self._h, _ptr(a)))
        return a

    def set_state(self, a):
        a = np.ascontiguousarray(a, dtype=np.float64).reshape(self.nz, self.ny, self.nx, 19)
        self._check(lib().dg_set_state(self._h, _ptr(a)))

    def copy_ddf(self):
        a = np.empty((self.nz + 2, self.ny + 2, self.nx + 2, 19), dtype=np.float64)
        self._check(lib().dg_copy_ddf(self._h, _ptr(a)))
        return a

    def dump(self, step):
        self._check(lib().dg_dump(self._h, step))

    def read_dump(self, step):
        self._check(lib().dg_read_dump(self._h, step))

    # macro / statistics
    def copy_vel(self):
        shape = (self.nz + 2, self.ny + 2, self.nx + 2)
        out = [np.empty(shape, dtype=np.float64) for _ in range(4)]
        self._check(lib().dg_copy_vel(self._h, *[_ptr(a) for a in out]))
        return out

    def stats_values(self):
        diag = np.empty(12, dtype=np.float64)
        prof = np.empty((self.nx, 9), dtype=np.float64)
        self._check(lib().dg_stats_values(self._h, _ptr(diag), _ptr(prof)))
        return diag, prof

    def stats(self, step):
        self._check(lib().dg_stats(self._h, step))

    def output_2d(self, step):
        self._check(lib().dg_output_2d(self._h, step))

    def stats_accumulate(self):
        self._check(lib().dg_stats_accumulate(self._h))

    def stats_accumulated(self):
        prof = np.empty((self.nx, 9), dtype=np.float64)
        n = ctypes.c_longlong(0)
        self._check(lib().dg_stats_accumulated(self._h, _ptr(prof), ctypes.byref(n)))
        return prof, n.value

    def stats_reset(self):
        self._check(lib().dg_stats_reset(self._h))

    def moments(self):
        m = np.empty(4, dtype=np.float64)
        self._check(lib().dg_moments(self._h, _ptr(m)))
        return m

    def mesh(self):
        xc = np.empty(self.nx + 2)
        dxx = np.empty(self.nx + 2)
        self._check(lib().dg_get_mesh(self._h, _ptr(xc), _ptr(dxx)))
        return xc, dxx

    # device-resident state in the engine's SoA layout (19 * pop_stride elements)
    @property
    def soa_len(self):
        return 19 * self.info.pop_stride

    def get_state_device(self, dst_ptr):
        self._check(lib().dg_get_state_device(self._h, ctypes.c_void_p(dst_ptr)))

    def set_state_device(self, src_ptr):
        self._check(lib().dg_set_state_device(self._h, ctypes.c_void_p(src_ptr)))

    def adjoint_step(self, istep, f_ptr, lam_next_ptr, lam_out_ptr):
        self._check(lib().dg_adjoint_step(self._h, istep, ctypes.c_void_p(f_ptr), ctypes.c_void_p(lam_next_ptr),
                                          ctypes.c_void_p(lam_out_ptr)))

    SPECTRAL_KEYS = ("te", "etotal", "ediss", "ediss_total", "eta", "vk", "tk", "uprm", "tmse", "retms", "xl",
                     "kmxeta", "skew", "flat")

    def spectral_stats(self, nbins=None):
        """(dict of the 14 values of dg_spectral_stats, shell spectrum E(k) for k = 0..nbins-1)."""
        nb = self.nx + 1 if nbins is None else int(nbins)
        vals = np.zeros(14)
        spec = np.zeros(max(nb, 1))
        self._check(lib().dg_spectral_stats(self._h, _ptr(vals), _ptr(spec), nb))
        return dict(zip(self.SPECTRAL_KEYS, vals.tolist())), spec[:nb]

    def output_spectral(self, step):
        self._check(lib().dg_output_spectral(self._h, step))

    def run_store(self, istep0, n, states_ptr, stride_bytes):
        self._check(lib().dg_run_store(self._h, istep0, n, ctypes.c_void_p(states_ptr), stride_bytes))

    def adjoint_run(self, istep0, n, states_ptr, stride_bytes, lam_ptr):
        self._check(lib().dg_adjoint_run(self._h, istep0, n, ctypes.c_void_p(states_ptr), stride_bytes,
                                         ctypes.c_void_p(lam_ptr)))

    def device_ptr(self, which):
        return lib().dg_device_ptr(self._h, which)

    # body-force field (extension): phi (nz, ny, nx) along `axis`; None removes it
    def set_force_field(self, axis, phi):
        if phi is None:
            self._check(lib().dg_set_force_field(self._h, 0, None))
            return
        a = np.ascontiguousarray(phi, dtype=np.float64)
        if a.shape != (self.nz, self.ny, self.nx):
            raise ValueError(f"force field shape {a.shape}, expected {(self.nz, self.ny, self.nx)}")
        self._check(lib().dg_set_force_field(self._h, int(axis), _ptr(a)))

    def field_grad(self, reset=False):
        """dJ/dphi accumulated by adjoint_step, shape (nz, ny, nx)."""
        out = np.empty((self.nz, self.ny, self.nx), dtype=np.float64)
        self._check(lib().dg_field_grad(self._h, _ptr(out), 1 if reset else 0))
        return out
