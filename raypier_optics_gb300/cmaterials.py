"""Interface materials and dispersion curves, mirroring
``raypier.core.cmaterials`` (cmaterials.pyx).

Each material packs itself into an ``rp_material`` record; the child-ray
evaluation (``eval_child_ray_c``) runs on the GPU inside the generation
kernel.  Dispersion curves are evaluated on the device once per scene upload
for every wavelength of the ray collection, as the reference's
``on_set_wavelengths`` does (cmaterials.pyx:883-887).
"""
from __future__ import annotations

import math

import numpy as np

from .ctracer import GaussletCollection, InterfaceMaterial, Ray

(MAT_NONE, MAT_OPAQUE, MAT_TRANSPARENT, MAT_PEC, MAT_PARTIAL, MAT_LINEAR_POLARISING, MAT_WAVEPLATE,
 MAT_DIELECTRIC, MAT_FULL_DIELECTRIC, MAT_FULL_DIELECTRIC_DISPERSIVE, MAT_CIRCULAR_APERTURE,
 MAT_RECT_APERTURE, MAT_SINGLE_LAYER_COATED, MAT_COATED_DISPERSIVE, MAT_DIFFRACTION_GRATING,
 MAT_RESAMPLE_GAUSSLET) = range(16)


def Convert_to_SP(ray, normal):
    """Project a ray's E-field onto the S/P basis of `normal`, on the GPU
    (convert_to_sp, cmaterials.pyx:49-101)."""
    from . import unitcalls
    return unitcalls.convert_to_sp([ray], [normal])[0]


class BaseDispersionCurve:
    """cmaterials.pyx:152-239.  formula_id 0 (constant), 1, 2 (Sellmeier) and 3
    (polynomial) are supported; 5 is rejected (the reference's sellmeier_5 has
    no return value)."""

    def __init__(self, formula_id, coefs, absorption=0.0, wavelength_min=0.1, wavelength_max=1000000.0):
        if formula_id not in (0, 1, 2, 3, 5):
            raise ValueError("Unknown formula id (%d)" % (formula_id,))
        self.coefs = np.ascontiguousarray(coefs, dtype=np.double)
        self.formula_id = int(formula_id)
        self.absorption = float(absorption)
        self.wavelength_min = float(wavelength_min)
        self.wavelength_max = float(wavelength_max)

    def _check_range(self, wavelen):
        for wvl in np.atleast_1d(wavelen):
            if (wvl < self.wavelength_min) or (wvl > self.wavelength_max):
                raise ValueError("Wavelength (%f) outside range of dispersion curve (%f -> %f)" % (
                    wvl, self.wavelength_min, self.wavelength_max))

    def evaluate_n(self, wavelen):
        """Complex refractive index for the given wavelengths (microns), on the GPU."""
        from . import unitcalls
        wl = np.atleast_1d(np.asarray(wavelen, dtype=np.double))
        self._check_range(wl)
        return unitcalls.dispersion_n(self, wl)


vacuum = BaseDispersionCurve(0, [1.0])


class OpaqueMaterial(InterfaceMaterial):
    """cmaterials.pyx:242-251: absorbs, no child."""
    type_code = MAT_OPAQUE

    def _pack(self, rec, tables):
        pass


class TransparentMaterial(InterfaceMaterial):
    """cmaterials.pyx:254-278"""
    type_code = MAT_TRANSPARENT

    def _pack(self, rec, tables):
        pass


class PECMaterial(InterfaceMaterial):
    """cmaterials.pyx:281-319: perfect reflector."""
    type_code = MAT_PEC

    def _pack(self, rec, tables):
        pass


class PartiallyReflectiveMaterial(InterfaceMaterial):
    """cmaterials.pyx:322-397"""
    type_code = MAT_PARTIAL

    def __init__(self, **kwds):
        super().__init__(**kwds)
        self.reflectivity = kwds.get("reflectivity", 0.5)

    @property
    def reflectivity(self):
        return self._reflectivity

    @reflectivity.setter
    def reflectivity(self, val):
        if val < 0.0 or val > 1.0:
            raise ValueError(f"Reflectivity must be in range 0.0 to 1.0 ({val} given).")
        self._reflectivity = float(val)

    def _pack(self, rec, tables):
        rec['p'][0] = self._reflectivity


class LinearPolarisingMaterial(InterfaceMaterial):
    """cmaterials.pyx:400-455"""
    type_code = MAT_LINEAR_POLARISING

    def _pack(self, rec, tables):
        pass


class WaveplateMaterial(InterfaceMaterial):
    """cmaterials.pyx:458-551; the retardance is stored as the unit complex
    number exp(2 pi i r) exactly as the reference's setter computes it."""
    type_code = MAT_WAVEPLATE

    def __init__(self, **kwds):
        super().__init__(**kwds)
        self.retardance = kwds.get("retardance", 0.25)
        self.fast_axis = kwds.get("fast_axis", (1.0, 0, 0))

    @property
    def retardance(self):
        val = math.atan2(self._ret_im, self._ret_re) / (2 * math.pi)
        if val < 0:
            val += 1.0
        return val

    @retardance.setter
    def retardance(self, val):
        self._ret_re = math.cos(val * 2 * math.pi)
        self._ret_im = math.sin(val * 2 * math.pi)

    @property
    def fast_axis(self):
        return self._fast_axis

    @fast_axis.setter
    def fast_axis(self, ax):
        self._fast_axis = (float(ax[0]), float(ax[1]), float(ax[2]))

    def apply_retardance(self, r):
        out = Ray()
        out.ray[()] = r.ray
        E1 = r.E1_amp
        out.E1_amp = complex(E1.real * self._ret_re - E1.imag * self._ret_im,
                             E1.imag * self._ret_re + E1.real * self._ret_im)
        return out

    def _pack(self, rec, tables):
        rec['p'][:5] = (self._ret_re, self._ret_im) + self._fast_axis


class DielectricMaterial(InterfaceMaterial):
    """cmaterials.pyx:554-724"""
    type_code = MAT_DIELECTRIC

    def __init__(self, **kwds):
        super().__init__(**kwds)
        self.n_inside = kwds.get('n_inside', 1.5)
        self.n_outside = kwds.get('n_outside', 1.0)

    @property
    def n_inside(self):
        return self._n_inside

    @n_inside.setter
    def n_inside(self, v):
        self._n_inside = complex(v)

    @property
    def n_outside(self):
        return self._n_outside

    @n_outside.setter
    def n_outside(self, v):
        self._n_outside = complex(v)

    def _pack(self, rec, tables):
        rec['n_inside'] = (self._n_inside.real, self._n_inside.imag)
        rec['n_outside'] = (self._n_outside.real, self._n_outside.imag)


class FullDielectricMaterial(DielectricMaterial):
    """cmaterials.pyx:727-872: complex Fresnel split into a reflected and a
    transmitted child, each kept when its power fraction exceeds its threshold."""
    type_code = MAT_FULL_DIELECTRIC

    def __init__(self, **kwds):
        super().__init__(**kwds)
        self.n_coating = kwds.get("n_coating", 1.0)
        self.thickness = kwds.get("thickness", 0.1)
        self.reflection_threshold = float(kwds.get('reflection_threshold', 0.1))
        self.transmission_threshold = float(kwds.get('transmission_threshold', 0.1))

    @property
    def n_coating(self):
        return self._n_coating

    @n_coating.setter
    def n_coating(self, v):
        self._n_coating = complex(v)

    def _pack(self, rec, tables):
        super()._pack(rec, tables)
        rec['reflection_threshold'] = self.reflection_threshold
        rec['transmission_threshold'] = self.transmission_threshold


class FullDielectricDispersiveMaterial(InterfaceMaterial):
    """cmaterials.pyx:875-1013"""
    type_code = MAT_FULL_DIELECTRIC_DISPERSIVE

    def __init__(self, **kwds):
        super().__init__(**kwds)
        self.dispersion_inside = kwds.get("dispersion_inside", vacuum)
        self.dispersion_outside = kwds.get("dispersion_outside", vacuum)
        self.reflection_threshold = float(kwds.get('reflection_threshold', 0.1))
        self.transmission_threshold = float(kwds.get('transmission_threshold', 0.1))

    def on_set_wavelengths(self):
        # the reference evaluates its n tables here and raises ValueError for a
        # wavelength out of range; the tables themselves are built on the device
        self.dispersion_inside._check_range(self._wavelengths)
        self.dispersion_outside._check_range(self._wavelengths)

    def _pack(self, rec, tables):
        rec['curve_inside'] = tables.add_dispersion(self.dispersion_inside)
        rec['curve_outside'] = tables.add_dispersion(self.dispersion_outside)
        rec['reflection_threshold'] = self.reflection_threshold
        rec['transmission_threshold'] = self.transmission_threshold


class SingleLayerCoatedMaterial(FullDielectricMaterial):
    """cmaterials.pyx:1017-1184: Fresnel coefficients of one thin film (index
    n_coating, thickness in microns) on the interface, by the reference's
    characteristic-matrix product; the ray's wavelength enters the film phase."""
    type_code = MAT_SINGLE_LAYER_COATED

    def _pack(self, rec, tables):
        super()._pack(rec, tables)
        c = complex(self.n_coating)
        rec['p'][:3] = (c.real, c.imag, float(self.thickness))


class CoatedDispersiveMaterial(InterfaceMaterial):
    """cmaterials.pyx:1187-1381: the single-layer coating with every index
    (inside, outside, coating) from a dispersion curve at the ray's wavelength."""
    type_code = MAT_COATED_DISPERSIVE

    def __init__(self, **kwds):
        super().__init__(**kwds)
        self.reflection_threshold = float(kwds.get('reflection_threshold', 0.1))
        self.transmission_threshold = float(kwds.get('transmission_threshold', 0.1))
        self.dispersion_inside = kwds.get("dispersion_inside", vacuum)
        self.dispersion_outside = kwds.get("dispersion_outside", vacuum)
        self.dispersion_coating = kwds.get("dispersion_coating", vacuum)
        self.coating_thickness = float(kwds.get("coating_thickness", 0.1))

    def on_set_wavelengths(self):
        self.dispersion_inside._check_range(self._wavelengths)
        self.dispersion_outside._check_range(self._wavelengths)
        self.dispersion_coating._check_range(self._wavelengths)

    def _pack(self, rec, tables):
        rec['curve_inside'] = tables.add_dispersion(self.dispersion_inside)
        rec['curve_outside'] = tables.add_dispersion(self.dispersion_outside)
        rec['p'][0] = float(tables.add_dispersion(self.dispersion_coating))
        rec['p'][1] = self.coating_thickness
        rec['reflection_threshold'] = self.reflection_threshold
        rec['transmission_threshold'] = self.transmission_threshold


class DiffractionGratingMaterial(InterfaceMaterial):
    """cmaterials.pyx:1437-1543: a reflective grating; the diffracted direction
    shifts the component along the face tangent by order * wavelength /
    (line spacing * n), and the grating phase depends on the offset from `origin`."""
    type_code = MAT_DIFFRACTION_GRATING

    def __init__(self, **kwds):
        super().__init__(**kwds)
        self.lines_per_mm = float(kwds.get("lines_per_mm", 1000))
        self.order = int(kwds.get("order", 1))
        self.efficiency = float(kwds.get("efficiency", 1.0))
        self.origin = tuple(map(float, kwds.get("origin", (0.0, 0.0, 0.0))))

    def _pack(self, rec, tables):
        rec['p'][:6] = (self.lines_per_mm, float(self.order), self.efficiency) + tuple(self.origin)


class CircularApertureMaterial(InterfaceMaterial):
    """cmaterials.pyx:1602-1662"""
    type_code = MAT_CIRCULAR_APERTURE

    def __init__(self, **kwds):
        super().__init__(**kwds)
        self.outer_radius = float(kwds.get("outer_radius", 25.0))
        self.radius = float(kwds.get("radius", 15.0))
        self.edge_width = float(kwds.get("edge_width", 1.0))
        self.origin = tuple(map(float, kwds.get("origin", (0.0, 0.0, 0.0))))
        self.invert = int(kwds.get("invert", 0))

    def _pack(self, rec, tables):
        rec['p'][:7] = (self.outer_radius, self.radius, self.edge_width, float(self.invert)) + tuple(self.origin)


class RectangularApertureMaterial(InterfaceMaterial):
    """cmaterials.pyx:1665-1763"""
    type_code = MAT_RECT_APERTURE

    def __init__(self, **kwds):
        super().__init__(**kwds)
        self.outer_width = float(kwds.get("outer_width", 15.0))
        self.outer_height = float(kwds.get("outer_height", 20.0))
        self.width = float(kwds.get("width", 5.0))
        self.height = float(kwds.get("height", 10.0))
        self.edge_width = float(kwds.get("edge_width", 1.0))
        self.origin = tuple(map(float, kwds.get("origin", (0.0, 0.0, 0.0))))
        self.invert = int(kwds.get("invert", 0))

    def _pack(self, rec, tables):
        rec['p'][:9] = (self.outer_width, self.outer_height, self.width, self.height, self.edge_width,
                        float(self.invert)) + tuple(self.origin)


class ResampleGaussletMaterial(InterfaceMaterial):
    """cmaterials.pyx:1766-1830: a decomposition pseudo-material.  During a
    Gausslet generation it captures every gausslet whose base ray carries the
    GAUSSLET bit; after the generation ``eval_func`` maps the captured
    GaussletCollection to new gausslets that are appended to the generation.
    It emits no child rays."""
    type_code = MAT_RESAMPLE_GAUSSLET

    def __init__(self, **kwds):
        super().__init__(**kwds)
        self.capture_count = 0
        self.captured_rays = GaussletCollection(kwds.get("size", 2))
        self._evaluation_func = None
        func = kwds.get("eval_func", None)
        if func is not None:
            self.eval_func = func

    @property
    def eval_func(self):
        return self._evaluation_func

    @eval_func.setter
    def eval_func(self, obj):
        if not callable(obj):
            raise ValueError("The eval_func property must be a callable.")
        self._evaluation_func = obj

    def is_decomp_material(self):
        return True

    def _pack(self, rec, tables):
        pass

    def eval_decomposed_rays(self, new_rays):
        """eval_decomposed_rays_c (cmaterials.pyx:1820-1830): appends
        eval_func(captured gausslets) to `new_rays` and clears the capture."""
        self.captured_rays.wavelengths = new_rays.wavelengths
        gc = self._evaluation_func(self.captured_rays)
        new_rays.extend(gc)
        self.captured_rays.clear_ray_list()
