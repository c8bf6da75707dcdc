"""ctypes binding of the oracle (liboracle.so): the CPU restatement of the
reference DUGKS step.  TEST INFRASTRUCTURE ONLY -- imported by tests/,
__graft_entry__.smoke() and bench.py's CPU-baseline legs as the checker.

Arrays: the oracle works on the reference's ghosted AoS layout,
shape (nz+2, ny+2, nx+2, 19); `to_ghosted` / `interior` convert from / to the
dump order (nz, ny, nx, 19) used by the engine's C ABI.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
_D = ctypes.POINTER(ctypes.c_double)
_F = ctypes.POINTER(ctypes.c_float)


class Cfg(ctypes.Structure):
    _fields_ = [("nx", ctypes.c_int), ("ny", ctypes.c_int), ("nz", ctypes.c_int), ("periodic_x", ctypes.c_int),
                ("mesh", ctypes.c_int), ("recon", ctypes.c_int), ("face_force", ctypes.c_int),
                ("perturb", ctypes.c_int), ("dx", ctypes.c_double), ("dy", ctypes.c_double),
                ("dz", ctypes.c_double), ("dt", ctypes.c_double), ("visc", ctypes.c_double),
                ("xwidth", ctypes.c_double), ("ywidth", ctypes.c_double), ("zwidth", ctypes.c_double),
                ("Fx", ctypes.c_double), ("Fy", ctypes.c_double), ("Fz", ctypes.c_double),
                ("xc", _D), ("dxx", _D)]


_lib = None


def build():
    subprocess.run(["make", "-s", "-C", HERE], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        P = ctypes.POINTER(Cfg)
        for sfx, T in (("f64", _D), ("f32", _F)):
            getattr(L, f"oracle_coefficients_{sfx}").argtypes = [P, _D]
            getattr(L, f"oracle_init_{sfx}").argtypes = [P, ctypes.c_int, T]
            getattr(L, f"oracle_init_case_{sfx}").argtypes = [P, ctypes.c_int, _D, T]
            getattr(L, f"oracle_fbar_{sfx}").argtypes = [P, T, T, ctypes.c_int, ctypes.c_int]
            getattr(L, f"oracle_run_{sfx}").argtypes = [P, T, ctypes.c_int, ctypes.c_int, ctypes.c_int]
            getattr(L, f"oracle_macro_{sfx}").argtypes = [P, T, T, T, T, T]
            getattr(L, f"oracle_stats_{sfx}").argtypes = [ctypes.c_int] * 3 + [T] * 4 + [_D, _D]
        L.oracle_max_threads.restype = ctypes.c_int
        _lib = L
    return _lib


class Oracle:
    """Reference step on the CPU for one configuration.

    Keeps numpy copies of the stretched-mesh arrays alive for the C struct."""

    def __init__(self, nx, ny, nz, dx, dy, dz, dt, visc, F=(0.0, 0.0, 0.0), periodic_x=0, xwidth=None,
                 ywidth=None, zwidth=None, xc=None, dxx=None, recon=0, face_force=0, perturb=0, dtype=np.float64):
        self.dtype = np.dtype(dtype)
        self.sfx = "f64" if self.dtype == np.float64 else "f32"
        self._xc = None if xc is None else np.ascontiguousarray(xc, dtype=np.float64)
        self._dxx = None if dxx is None else np.ascontiguousarray(dxx, dtype=np.float64)
        c = Cfg()
        c.nx, c.ny, c.nz = nx, ny, nz
        c.periodic_x = periodic_x
        c.mesh = 1 if xc is not None else 0
        c.recon, c.face_force, c.perturb = recon, face_force, perturb
        c.dx, c.dy, c.dz, c.dt, c.visc = dx, dy, dz, dt, visc
        c.xwidth = xwidth if xwidth is not None else dx * nx
        c.ywidth = ywidth if ywidth is not None else dy * ny
        c.zwidth = zwidth if zwidth is not None else dz * nz
        c.Fx, c.Fy, c.Fz = F
        if self._xc is not None:
            c.xc = self._xc.ctypes.data_as(_D)
            c.dxx = self._dxx.ctypes.data_as(_D)
        self.cfg = c
        self.shape = (nz + 2, ny + 2, nx + 2, 19)

    @classmethod
    def from_config(cls, text, dtype=np.float64, workdir=".", **kw):
        """The oracle of a config.txt text, set up from the text alone (nothing
        of the engine): reference keys parsed as src/config.h and
        src/numerics.cu:62-106 do (std::stof / std::stoi), dx, dy, dz and dt in
        the reference's `real`, and for the extension key mesh=tanh|file the
        stretched mesh of src/fortran/channel (faces from run/mesh.py:21-25 or
        from the mesh file, centres, widths and ghosts as dugks.cuf:107-121,
        dt from the first cell width as dugks.cuf:138)."""
        c = setup_from_config(text, dtype=dtype, workdir=workdir)
        kw.setdefault("recon", 1 if c["kv"].get("recon") == "gradient" else 0)
        o = cls(c["nx"], c["ny"], c["nz"], c["dx"], c["dy"], c["dz"], c["dt"], c["visc"], F=c["F"],
                periodic_x=c["periodic_x"], xwidth=c["xwidth"], ywidth=c["ywidth"], zwidth=c["zwidth"],
                xc=c["xc"], dxx=c["dxx"], perturb=c["perturb"], dtype=dtype, **kw)
        o.setup = c
        return o

    def initial_state(self):
        """Initial state (dump order) of the case the config names: tg_eq (with the
        extension key tg_u0), channel, or the seeded channel_turb start."""
        c = self.setup
        kv = c["kv"]
        kind = self.CASE_KIND[c["case"]]
        if kind == 0:
            par = (_double(kv.get("tg_u0", "0.1")),)
        elif kind == 2:
            par = (_double(kv.get("ub", "0.1")), _double(kv.get("re_tau", "180")), _double(kv.get("pert_amp", "0.1")),
                   _double(kv.get("streak_amp", "0.05")), _stoi(kv.get("seed", "0")), _stoi(kv.get("streak_m", "4")))
        else:
            par = ()
        return interior(self.init_case(kind, par))

    @classmethod
    def from_engine_info(cls, info, xc=None, dxx=None, dtype=np.float64, **kw):
        F = tuple(info.ambient)
        return cls(info.nx, info.ny, info.nz, info.dx, info.dy, info.dz, info.dt, info.visc, F=F,
                   periodic_x=info.periodic[0], xwidth=info.xwidth, ywidth=info.ywidth, zwidth=info.zwidth,
                   xc=xc if info.mesh else None, dxx=dxx if info.mesh else None, perturb=info.perturb,
                   dtype=dtype, **kw)

    def _p(self, a):
        assert a.dtype == self.dtype and a.flags.c_contiguous
        return a.ctypes.data_as(_D if self.sfx == "f64" else _F)

    def coefficients(self):
        out = np.empty(13)
        getattr(lib(), f"oracle_coefficients_{self.sfx}")(ctypes.byref(self.cfg), out.ctypes.data_as(_D))
        return out

    def init(self, kind):
        f = np.zeros(self.shape, dtype=self.dtype)
        rc = getattr(lib(), f"oracle_init_{self.sfx}")(ctypes.byref(self.cfg), kind, self._p(f))
        assert rc == 0
        return f

    CASE_KIND = {"tg_eq": 0, "channel": 1, "channel_turb": 2}

    def init_case(self, kind, par=()):
        """Initial state of case `kind` (0 tg_eq with amplitude par[0], 1 channel,
        2 the seeded turbulent-channel start, par = (ub, re_tau, amp, streak, seed, m))
        on the interior of a ghosted box."""
        f = np.zeros(self.shape, dtype=self.dtype)
        p = np.zeros(8)
        p[:len(par)] = par
        rc = getattr(lib(), f"oracle_init_case_{self.sfx}")(ctypes.byref(self.cfg), kind, p.ctypes.data_as(_D),
                                                           self._p(f))
        assert rc == 0
        return f

    def fbar(self, f, step=1, nthreads=0):
        fb = np.zeros(self.shape, dtype=self.dtype)
        rc = getattr(lib(), f"oracle_fbar_{self.sfx}")(ctypes.byref(self.cfg), self._p(f), self._p(fb), step,
                                                       nthreads)
        assert rc == 0, rc
        return fb

    def run(self, f, istep0, nsteps, nthreads=0):
        """Advance the ghosted state f in place."""
        rc = getattr(lib(), f"oracle_run_{self.sfx}")(ctypes.byref(self.cfg), self._p(f), istep0, nsteps, nthreads)
        assert rc == 0, rc
        return f

    def tangent_run(self, f, df, istep0, nsteps, nthreads=0):
        """Forward-mode tangent of nsteps steps (FP64): f <- S^n(f) and
        df <- dS^n(f)[df] in place, both ghosted (liboracle's restatement run on
        dual numbers, libtangent.so)."""
        assert self.sfx == "f64"
        for a in (f, df):
            assert a.dtype == np.float64 and a.flags.c_contiguous and a.shape == self.shape
        rc = tangent_lib().oracle_tangent_run(ctypes.byref(self.cfg), f.ctypes.data_as(_D), df.ctypes.data_as(_D),
                                              istep0, nsteps, nthreads)
        assert rc == 0, rc
        return f, df

    def macro(self, f):
        out = [np.zeros(self.shape[:3], dtype=self.dtype) for _ in range(4)]
        getattr(lib(), f"oracle_macro_{self.sfx}")(ctypes.byref(self.cfg), self._p(f), *[self._p(a) for a in out])
        return out

    def stats(self, f):
        """statistics_serial on the macro fields of f: (diag[12], prof[nx, 9])."""
        rho, ux, uy, uz = [np.ascontiguousarray(a[1:-1, 1:-1, 1:-1]) for a in self.macro(f)]
        diag = np.empty(12)
        prof = np.empty((self.cfg.nx, 9))
        getattr(lib(), f"oracle_stats_{self.sfx}")(self.cfg.nx, self.cfg.ny, self.cfg.nz, self._p(rho),
                                                   self._p(ux), self._p(uy), self._p(uz),
                                                   diag.ctypes.data_as(_D), prof.ctypes.data_as(_D))
        return diag, prof


# ---------------------------------------------------------------------------
# configuration and mesh, restated from the reference (independent of the engine)
# ---------------------------------------------------------------------------
_libc = None


def _c():
    global _libc
    if _libc is None:
        _libc = ctypes.CDLL(None)
        _libc.strtof.restype = ctypes.c_float
        _libc.strtof.argtypes = [ctypes.c_char_p, ctypes.POINTER(ctypes.c_char_p)]
        _libc.strtod.restype = ctypes.c_double
        _libc.strtod.argtypes = [ctypes.c_char_p, ctypes.POINTER(ctypes.c_char_p)]
        _libc.strtol.restype = ctypes.c_long
        _libc.strtol.argtypes = [ctypes.c_char_p, ctypes.POINTER(ctypes.c_char_p), ctypes.c_int]
    return _libc


def _stof(v):
    """std::stof (strtof: the value rounded to float once), widened."""
    return float(_c().strtof(v.encode(), None))


def _double(v):
    return float(_c().strtod(v.encode(), None))


def _stoi(v):
    return int(_c().strtol(v.encode(), None, 10))


def parse_config(text):
    """key -> value of config.txt text with src/config.h:17-74's rules: lines split
    at '=', the second field is the value, lines without '=' are ignored, no
    trimming, the first occurrence of a key wins."""
    kv = {}
    for line in text.split("\n"):
        parts = line.split("=")
        if len(parts) > 1 and parts[0] not in kv:
            kv[parts[0]] = parts[1]
    return kv


def tanh_faces(nx, L, alpha):
    """nx+1 face positions of the tanh wall-normal mesh, src/fortran/channel/run/mesh.py:21-25."""
    eta = -1.0 + 2.0 * np.arange(nx + 1, dtype=np.float64) / nx
    return L / (2.0 * alpha) * np.tanh(eta * 0.5 * (np.log(1.0 + alpha) - np.log(1.0 - alpha))) + 0.5 * L


def mesh_from_faces(xf, xwidth):
    """Cell centres and widths 0..nx+1 with the mirrored ghosts,
    src/fortran/channel/src/dugks.cuf:114-121."""
    xf = np.asarray(xf, dtype=np.float64)
    nx = len(xf) - 1
    xc = np.zeros(nx + 2)
    dxx = np.zeros(nx + 2)
    xc[1:nx + 1] = 0.5 * (xf[1:] + xf[:-1])
    dxx[1:nx + 1] = xf[1:] - xf[:-1]
    xc[0] = -xc[1]
    xc[nx + 1] = 2 * xwidth - xc[nx]
    dxx[0] = dxx[1]
    dxx[nx + 1] = dxx[nx]
    return xc, dxx


def setup_from_config(text, dtype=np.float64, workdir="."):
    """Grid, coefficients and mesh of a config text, computed here from the
    reference's formulas (src/numerics.cu:74-105 in `real` = dtype;
    the stretched mesh in double precision as the -r8 Fortran channel)."""
    kv = parse_config(text)
    R = np.float64 if np.dtype(dtype) == np.float64 else np.float32
    nx, ny, nz = (_stoi(kv[k]) for k in ("nx", "ny", "nz"))
    cfl, xw, yw, zw, visc = (R(_stof(kv[k])) for k in ("CFL", "xwidth", "ywidth", "zwidth", "visc"))
    F = tuple(float(R(_stof(kv[k]))) for k in ("ambient_fx", "ambient_fy", "ambient_fz"))
    RT = R(1.0 / 3.0)
    dx, dy, dz = xw / R(nx), yw / R(ny), zw / R(nz)
    mesh = kv.get("mesh", "uniform")
    xc = dxx = None
    if mesh in ("tanh", "file"):
        xw_d = _double(kv["xwidth"])
        if mesh == "tanh":
            xf = tanh_faces(nx, xw_d, _double(kv.get("mesh_alpha", "0.85")))
        else:
            path = kv.get("mesh_file", "mesh.txt")
            if not os.path.isabs(path):
                path = os.path.join(workdir, path)
            xf = np.array(open(path).read().split()[:nx + 1], dtype=np.float64)
        xc, dxx = mesh_from_faces(xf, xw_d)
        dt = cfl * R(dxx[1]) / np.sqrt(R(6) * RT)
    else:
        dt = cfl * dx / np.sqrt(R(6) * RT)
    return dict(kv=kv, case=kv["case"], nx=nx, ny=ny, nz=nz, dx=float(dx), dy=float(dy), dz=float(dz),
                dt=float(dt), visc=float(visc), F=F, xwidth=float(xw), ywidth=float(yw), zwidth=float(zw),
                periodic_x=_stoi(kv["periods_x"]), perturb=_stoi(kv["perturb"]), xc=xc, dxx=dxx)


_tan = None


def tangent_lib():
    global _tan
    if _tan is None:
        path = os.path.join(HERE, "libtangent.so")
        if not os.path.exists(path):
            build()
        L = ctypes.CDLL(path)
        L.oracle_tangent_run.argtypes = [ctypes.POINTER(Cfg), _D, _D, ctypes.c_int, ctypes.c_int, ctypes.c_int]
        _tan = L
    return _tan


def to_ghosted(f_dump, dtype=np.float64):
    nz, ny, nx, _ = f_dump.shape
    g = np.zeros((nz + 2, ny + 2, nx + 2, 19), dtype=dtype)
    g[1:-1, 1:-1, 1:-1] = f_dump
    return g


def interior(f_ghosted):
    return np.ascontiguousarray(f_ghosted[1:-1, 1:-1, 1:-1])


def max_threads():
    return lib().oracle_max_threads()


# ---------------------------------------------------------------------------
# The reference's own GPU kernels (oracle/_ref/*.cubin, launched by
# oracle/ref_runner.cpp).  Needs a GPU and the cubins built by build_ref.sh.
# ---------------------------------------------------------------------------
REF_LIB = os.path.join(HERE, "libref_runner.so")
REF_CUBIN = {0: os.path.join(HERE, "_ref", "dugks_f64.cubin"), 1: os.path.join(HERE, "_ref", "dugks_f32.cubin")}


class RefCfg(ctypes.Structure):
    _fields_ = [("nx", ctypes.c_int), ("ny", ctypes.c_int), ("nz", ctypes.c_int), ("periods", ctypes.c_int * 3),
                ("perturb", ctypes.c_int), ("recon", ctypes.c_int), ("CFL", ctypes.c_double),
                ("xwidth", ctypes.c_double), ("ywidth", ctypes.c_double), ("zwidth", ctypes.c_double),
                ("visc", ctypes.c_double), ("F", ctypes.c_double * 3)]


_ref = None


def ref_cubins_present():
    return all(os.path.exists(p) for p in REF_CUBIN.values())


def ref_lib():
    global _ref
    if _ref is None:
        if not os.path.exists(REF_LIB):
            build()
        L = ctypes.CDLL(REF_LIB)
        L.ref_open.argtypes = [ctypes.c_char_p, ctypes.c_int]
        L.ref_run.argtypes = [ctypes.c_int, ctypes.POINTER(RefCfg), _D, ctypes.c_int, ctypes.c_int, _D]
        L.ref_last_error.restype = ctypes.c_char_p
        _ref = L
    return _ref


def ref_run(f_ghosted, nx, ny, nz, CFL, xwidth, ywidth, zwidth, visc, F, periods=(0, 1, 1), istep0=1, nsteps=1,
            prec=0, perturb=0, recon=0):
    """Advance the ghosted double state in place with the reference's kernels;
    returns the CUDA-event milliseconds per step."""
    L = ref_lib()
    rc = L.ref_open(REF_CUBIN[prec].encode(), prec)
    if rc:
        raise RuntimeError(f"ref_open: {L.ref_last_error().decode()}")
    c = RefCfg()
    c.nx, c.ny, c.nz = nx, ny, nz
    c.periods[:] = list(periods)
    c.perturb, c.recon = perturb, recon
    c.CFL, c.xwidth, c.ywidth, c.zwidth, c.visc = CFL, xwidth, ywidth, zwidth, visc
    c.F[:] = list(F)
    assert f_ghosted.dtype == np.float64 and f_ghosted.flags.c_contiguous
    ms = ctypes.c_double(0)
    rc = L.ref_run(prec, ctypes.byref(c), f_ghosted.ctypes.data_as(_D), istep0, nsteps, ctypes.byref(ms))
    if rc:
        raise RuntimeError(f"ref_run: {L.ref_last_error().decode()}")
    return ms.value
