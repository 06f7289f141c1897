"""Surface distortions, mirroring ``raypier.core.cdistortions``
(cdistortions.pyx).  Zernike polynomials use ANSI ``j`` indexing
(cdistortions.pyx:104-136); evaluation runs on the GPU."""
from __future__ import annotations

import math

import numpy as np

from .ctracer import Distortion

DIST_ZERNIKE, DIST_SIMPLE_J7 = 1, 2


def eval_nmk(j):
    """ANSI index j -> (n, m, k) of a Zernike term (cdistortions.pyx:104-141).

    The terms of radial order n take the indices n(n+1)/2 .. n(n+3)/2, so n is
    the largest integer with n(n+1)/2 <= j and the azimuthal order follows
    from j = (n(n+2) + m)/2.  k is the slot of the radial polynomial R_n^|m|
    in the evaluation workspace, (n//2)(n//2 + 1) + |m|."""
    j = int(j)
    if j < 0:
        raise ValueError("J must be non-negative")
    n = (math.isqrt(8 * j + 1) - 1) // 2
    m = 2 * j - n * (n + 2)
    h = n // 2
    return (n, m, h * (h + 1) + abs(m))


zcoefs_dtype = np.dtype([('j', np.int32), ('n', np.int32), ('m', np.int32), ('k', np.int32), ('value', np.double)])


class SimpleTestZernikeJ7(Distortion):
    """cdistortions.pyx:39-81"""
    type_code = DIST_SIMPLE_J7

    def __init__(self, **kwds):
        self.unit_radius = float(kwds.get("unit_radius", 1.0))
        self.amplitude = float(kwds.get("amplitude", 1.0))

    def _pack(self, rec, tables):
        rec['type'] = DIST_SIMPLE_J7
        rec['unit_radius'] = self.unit_radius
        rec['amplitude'] = self.amplitude

    def z_offset_and_gradient(self, x, y):
        from . import unitcalls
        return unitcalls.distortion_eval(self, x, y)[:, :3]

    def z_offset(self, x, y):
        from . import unitcalls
        return unitcalls.distortion_eval(self, x, y)[:, 3]


class ZernikeDistortion(Distortion):
    """cdistortions.pyx:323-514.  Coefficients are given as ``j<N>=value``
    keywords or as a list of (j, value) pairs; they are held sorted by j."""
    type_code = DIST_ZERNIKE

    def __init__(self, *args, **coefs):
        self.coef_map = {}
        self.unit_radius = float(coefs.get("unit_radius", 1.0))
        cdict = {int(k[1:]): float(v) for k, v in coefs.items() if k.startswith("j")}
        if args:
            for k, v in args[0]:
                cdict[int(k)] = float(v)
        self.k_max = 0
        self.set_coefs(list(cdict.items()))

    def set_coefs(self, coefs):
        clist = sorted(coefs)
        self.j_max = max(j for j, v in clist)
        self.n_coefs = len(clist)
        self.coefs = np.empty(len(clist), dtype=zcoefs_dtype)
        n_max = 0
        self.coef_map = {}
        for i, (j, v) in enumerate(clist):
            n, m, k = eval_nmk(j)
            self.coef_map[j] = i
            self.coefs[i] = (j, n, m, k, v)
            n_max = max(n_max, n)
        k_max = (n_max // 2) * (n_max // 2 + 1) + n_max + 1
        if k_max > self.k_max:
            self.k_max = k_max

    def __getitem__(self, idx):
        if idx >= self.n_coefs:
            raise IndexError(f"Index {idx} greater than number of coeffs ({self.n_coefs}).")
        c = self.coefs[idx]
        return (int(c['j']), int(c['n']), int(c['m']), int(c['k']), float(c['value']))

    def __len__(self):
        return self.n_coefs

    def update_coef(self, j, value):
        try:
            i = self.coef_map[j]
            self.coefs[i]['value'] = value
        except KeyError:
            self.append_coef(j, value)

    def get_coef(self, j):
        return float(self.coefs[self.coef_map[j]]['value'])

    def append_coef(self, k, value):
        raise NotImplementedError()

    def _pack(self, rec, tables):
        if self.k_max > 48:
            raise NotImplementedError("Zernike orders above n=8 are not supported on the device")
        rec['type'] = DIST_ZERNIKE
        rec['n_coefs'] = self.n_coefs
        rec['k_max'] = self.k_max
        flat = np.stack([self.coefs['j'], self.coefs['n'], self.coefs['m'], self.coefs['k'],
                         self.coefs['value']], axis=1).astype(np.double)
        rec['aux'] = tables.add_aux(flat.reshape(-1))
        rec['unit_radius'] = self.unit_radius
        rec['amplitude'] = 1.0

    def z_offset_and_gradient(self, x, y):
        from . import unitcalls
        return unitcalls.distortion_eval(self, x, y)[:, :3]

    def z_offset(self, x, y):
        from . import unitcalls
        return unitcalls.distortion_eval(self, x, y)[:, 3]
