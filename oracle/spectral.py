"""CPU restatement (numpy, FP64) of the reference's spectral statistics of a
periodic box, src/fortran/dhit/src/stat.f90:5-205 (subroutine stat_te) with
the velocity of src/fortran/dhit/src/main.cuf:86-103.

Test infrastructure: the checker of dg_spectral_stats in tests/, never part
of the product.  The reference keeps velocities, spectra and sums in single
precision around double-precision FFTs; this restatement (like the engine)
computes everything in FP64 with the reference's constants (pi = 3.14159 in
single precision, stat.f90:28; wavenumbers 2 pi / xwidth along every axis,
stat.f90:85-106).
"""
import numpy as np

PI = float(np.float32(3.14159))
KEYS = ("te", "etotal", "ediss", "ediss_total", "eta", "vk", "tk", "uprm", "tmse", "retms", "xl", "kmxeta",
        "skew", "flat")


def velocity(f):
    """u = j / rho per cell of a state in dump order (nz, ny, nx, 19), main.cuf:86-103."""
    c = np.array([[0, 0, 0], [1, 0, 0], [-1, 0, 0], [0, 1, 0], [0, -1, 0], [0, 0, 1], [0, 0, -1],
                  [1, 1, 0], [-1, 1, 0], [1, -1, 0], [-1, -1, 0], [1, 0, 1], [-1, 0, 1], [1, 0, -1],
                  [-1, 0, -1], [0, 1, 1], [0, -1, 1], [0, 1, -1], [0, -1, -1]], dtype=np.float64)
    rho = f.sum(axis=-1)
    return tuple((f @ c[:, a]) / rho for a in range(3))


def freqs(n):
    """Signed integer frequencies of the FFT indices (the kx array, stat.f90:85-106)."""
    i = np.arange(n)
    return np.where(i < n // 2, i, i - n)


def stat_te(u, v, w, xwidth, visc):
    """The 14 values (KEYS) and the shell spectrum E(k), k = 0 .. 2 nx, of
    velocity fields u, v, w of shape (nz, ny, nx) (x fastest)."""
    nz, ny, nx = u.shape
    n = u.size
    te = 0.5 * np.sum(u * u + v * v + w * w) / n                        # stat.f90:60
    fx, fy, fz = freqs(nx)[None, None, :], freqs(ny)[None, :, None], freqs(nz)[:, None, None]
    ks = 2 * PI / xwidth
    ksqr = (ks * fx) ** 2 + (ks * fy) ** 2 + (ks * fz) ** 2
    hat = [np.fft.fftn(a - a.mean()) / n for a in (u, v, w)]           # stat.f90:66-73, 123-130
    et = 0.5 * sum((h * np.conj(h)).real for h in hat)                  # stat.f90:131
    ets = 2 * visc * et * ksqr                                          # stat.f90:132
    wn = np.rint(np.sqrt(fx * fx + fy * fy + fz * fz)).astype(int)     # (nz, ny, nx)
    ett = np.bincount(wn.ravel(), weights=et.ravel(), minlength=2 * nx + 1)   # stat.f90:142-151
    etts = np.bincount(wn.ravel(), weights=ets.ravel(), minlength=2 * nx + 1)
    etotal, ediss = ett.sum(), etts.sum()
    dx, cw = xwidth / nx, xwidth
    eta = (visc ** 3 / ediss) ** 0.25                                   # stat.f90:160-167
    vk = (visc * ediss) ** 0.25
    tk = np.sqrt(visc / ediss)
    uprm = np.sqrt(2.0 / 3.0 * etotal)
    tmse = np.sqrt(15 * visc * uprm ** 2 / ediss)
    retms = uprm * tmse / visc
    xl = uprm ** 3 / ediss
    kmxeta = (cw / 2 - 1.5 * dx) * (2 * PI) / cw * eta
    # longitudinal derivatives (stat.f90:176-190)
    d = [np.fft.ifftn(1j * ks * k * h).real * n for h, k in zip(hat, (fx, fy, fz))]
    bottom = sum(np.sum(x ** 2) for x in d) / (3 * n)
    skew = sum(np.sum(x ** 3) for x in d) / (3 * n) / bottom ** 1.5
    flat = sum(np.sum(x ** 4) for x in d) / (3 * n) / bottom ** 2
    vals = dict(zip(KEYS, (te, etotal, ediss, 0.0, eta, vk, tk, uprm, tmse, retms, xl, kmxeta, skew, flat)))
    return vals, ett
