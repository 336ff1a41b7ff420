"""Geometry descriptors, mirroring curadon's ``FanGeometry`` and
``ConeGeometry`` (python/standalone/src/curadon/geometry.py:53-336).

Same constructor arguments, attributes, validation messages and ASTRA-like
vector helpers as the reference.  Differences:

* the device plan is built on first use of ``.plan`` (construction needs no
  GPU); ``ConeGeometry`` also holds a plan, so per-view geometry is uploaded
  once instead of on every call;
* a scalar ``DSO`` is replaced by ``DSD`` exactly as the reference does
  (geometry.py:165) so that results stay identical for the same arguments;
  pass per-view arrays to use a scalar DSO.
"""
from __future__ import annotations

from typing import Any, List, Optional, Tuple, Union

import numpy as np

__all__ = ["FanGeometry", "FanVecGeometry", "ConeGeometry", "geom_to_str",
           "is_convertible_to_float"]


def is_convertible_to_float(val: Any) -> bool:
    try:
        float(val)
        return True
    except (ValueError, TypeError):
        return False


def geom_to_str(geom) -> str:
    """Human-readable summary (geometry.py:21-50)."""
    p = ["-----", "Geometry parameters",
         f"Distance from source to detector (DSD) = {geom.DSD}",
         f"Distance from source to origin (DSO) = {geom.DSO}"]
    if isinstance(geom, FanGeometry):
        p.append(f"Projections angles = {np.rad2deg(geom.angles)}")
    p += ["-----", "Detector parameters",
          f"Number of pixels (det_shape) = {geom.det_shape}",
          f"Size of each pixel (det_spacing) = {geom.det_spacing}",
          f"Total size of the detector (det_size) = {np.asarray(geom.det_shape) * geom.det_spacing}",
          f"Detector rotation (det_rotation) = {geom.det_rotation}",
          f"Offset of detector (det_offset) = {geom.det_offset}",
          "-----", "Image parameters",
          f"Number of voxels (vol_shape) = {geom.vol_shape}",
          f"Size of each voxel (vol_spacing) = {geom.vol_spacing}",
          f"Total size of the image (vol_size) = {geom.vol_shape * geom.vol_spacing}",
          f"Offset of image from origin (vol_offset) = {geom.vol_offset}"]
    return "\n".join(p)


class FanGeometry:
    """2D fan-beam geometry with per-view DSO/DSD (geometry.py:53-234)."""

    def __init__(self, DSD: Union[float, List[float]], DSO: Union[float, List[float]],
                 angles: List[float], vol_shape: Tuple[int, int], det_shape: int,
                 det_spacing: Optional[float] = None, det_offset: Optional[float] = None,
                 det_rotation: Optional[float] = None,
                 vol_spacing: Optional[Tuple[float, float]] = None,
                 vol_offset: Optional[Tuple[float, float]] = None, device: int = 0,
                 vol_prec: int = 32, sino_prec: int = 32):
        self.angles = np.asarray(angles)
        if self.angles.ndim != 1:
            raise AttributeError(f"Angles must be 1D array, got {str(self.angles.shape)}")
        self.nangles = self.angles.shape[0]

        if is_convertible_to_float(DSD):
            self.DSD = np.full(self.nangles, DSD)
        else:
            self.DSD = np.asarray(DSD)
            if self.DSD.ndim != 1 or self.DSD.size != self.nangles:
                raise AttributeError(
                    f"DSD must be a single float, or a list of floats nangles entries "
                    f"(is {self.DSD.size}, expected {self.nangles})")

        if is_convertible_to_float(DSO):
            # the reference fills a scalar DSO with DSD (geometry.py:165)
            self.DSO = np.full(self.nangles, DSD)
        else:
            self.DSO = np.asarray(DSO)
            if self.DSO.ndim != 1 or self.DSO.size != self.nangles:
                raise AttributeError(
                    f"DSO must be a single float, or a list of floats nangles entries "
                    f"(is {self.DSO.size}, expected {self.nangles})")

        self.vol_shape = np.asarray(vol_shape)
        if self.vol_shape.shape != (2,):
            raise AttributeError(f"vol_shape must be two values, got {str(self.vol_shape.shape)}")

        if not is_convertible_to_float(det_shape):
            raise AttributeError(f"det_shape must to be float, got {type(det_shape)}")
        self.det_shape = int(det_shape)

        self.det_spacing = self._scalar(det_spacing, "det_spacing", 1.0)
        self.det_offset = self._scalar(det_offset, "det_offset", 0.0)
        self.det_rotation = self._scalar(det_rotation, "det_rotation", 0.0)

        if vol_spacing is not None:
            self.vol_spacing = np.asarray(vol_spacing)
            if self.vol_spacing.shape != (2,):
                raise AttributeError(
                    f"vol_spacing must be two values, got {str(self.vol_spacing.shape)}")
        else:
            self.vol_spacing = np.ones(self.vol_shape.shape)

        if vol_offset is not None:
            self.vol_offset = np.asarray(vol_offset)
            if self.vol_offset.shape != (2,):
                raise AttributeError(
                    f"vol_offset must be two values, got {str(self.vol_offset.shape)}")
        else:
            self.vol_offset = np.zeros(self.vol_shape.shape)

        self.device = int(device)
        self.vol_prec = int(vol_prec)
        self.sino_prec = int(sino_prec)
        self._plan = None
        self._exact_plan = None

    @staticmethod
    def _scalar(v, name, default):
        if v is None:
            return float(default)
        if not is_convertible_to_float(v):
            raise TypeError(f"Expected {name} to be float, got {type(v)}")
        return float(v)

    def _make_plan(self):
        from .backend import plan_2d

        # COR is ignored by the reference's 2D path (geometry.py:226-228)
        return plan_2d(self.device, self.vol_prec, self.vol_shape, self.vol_spacing,
                       self.vol_offset, self.sino_prec, self.det_shape, self.det_spacing,
                       self.det_offset, self.DSO, self.DSD, self.angles, self.det_rotation, 0)

    @property
    def plan(self):
        """The device plan (``backend.plan_2d``), built on first use."""
        if self._plan is None:
            self._plan = self._make_plan()
        return self._plan

    @property
    def exact_plan(self):
        """A second plan whose forward filters in FP32 (algorithm "registers"),
        so that it and ``adjoint`` are exact transposes (matched gradients)."""
        if self._exact_plan is None:
            self._exact_plan = self._make_plan()
            self._exact_plan.set_algorithm(forward="registers")
        return self._exact_plan

    def to_vec(self):
        """ASTRA-like per-view vectors [src.x, src.y, det.x, det.y, u.x, u.y]
        (geometry.py:54-82)."""
        vecs = []
        for alpha, dsd, dso in zip(self.angles, self.DSD, self.DSO):
            cs, sn = np.cos(alpha), np.sin(alpha)
            R = np.asarray([[cs, sn], [-sn, cs]])
            src = R @ np.array([0.0, dso])
            det = R @ np.array([0.0, -(dsd - dso)])
            u = R @ np.array([1.0, 0.0])
            vecs.append([*src.tolist(), *det.tolist(), *u.tolist()])
        return vecs

    @staticmethod
    def from_vec(vol_shape: Tuple[int, int], det_shape: int, vecs: List[List[float]],
                 lossless: bool = False, **kwargs):
        """FanGeometry from ASTRA-like vectors (geometry.py:84-134): keeps the
        angle, |src| and |src - det| of each view and one detector spacing.
        ``lossless=True`` (an addition) keeps the vectors themselves instead
        (``FanVecGeometry``)."""
        if lossless:
            return FanVecGeometry(vol_shape, det_shape, vecs, **kwargs)
        vecs = np.asarray(vecs, dtype=np.float64)
        det_spacing = float(np.linalg.norm(vecs[0][-2:]))
        dsd, dso, angles = [], [], []
        for v in vecs:
            sx, sy, dx, dy, ux, uy = v
            src, det = np.asarray([sx, sy]), np.asarray([dx, dy])
            src2det = src - det
            dsd.append(np.linalg.norm(src2det))
            dso.append(np.linalg.norm(src))
            angles.append(np.arctan2(*src2det) % (2 * np.pi))
            if not np.isclose(det_spacing, np.linalg.norm([ux, uy])):
                raise AttributeError("Detector must have equal spacing for all projections")
        return FanGeometry(DSD=dsd, DSO=dso, angles=angles, vol_shape=vol_shape,
                           det_shape=det_shape, det_spacing=det_spacing, **kwargs)

    def sinogram_shape(self):
        return (self.nangles, self.det_shape)

    def __str__(self):
        return geom_to_str(self)


class FanVecGeometry(FanGeometry):
    """2D fan-beam geometry given by per-view vectors, kept as given.

    ``vecs`` is (nangles, 6): [source.x, source.y, detector.x, detector.y,
    u.x, u.y] in the world frame of ``FanGeometry.to_vec`` (x along the
    volume's width), with ``u`` the step from one detector cell centre to the
    next (its length is the detector spacing, equal for all views).  The
    reference's ``from_vec`` reduces such vectors to angles / DSO / DSD and so
    loses per-view shifts of source and detector (e.g. calibrated or jittered
    trajectories); here the plan uses the vectors themselves
    (``cg_plan2d_create_vec``).  ``angles``, ``DSO``, ``DSD`` and
    ``det_spacing`` hold that reduction for information."""

    def __init__(self, vol_shape: Tuple[int, int], det_shape: int, vecs,
                 vol_spacing: Optional[Tuple[float, float]] = None,
                 vol_offset: Optional[Tuple[float, float]] = None, device: int = 0,
                 vol_prec: int = 32, sino_prec: int = 32):
        v = np.asarray(vecs, dtype=np.float64)
        if v.ndim != 2 or v.shape[1] != 6 or v.shape[0] == 0:
            raise AttributeError(f"vecs must be (nangles, 6), got {v.shape}")
        reduced = FanGeometry.from_vec(vol_shape, det_shape, v, vol_spacing=vol_spacing,
                                       vol_offset=vol_offset, device=device, vol_prec=vol_prec,
                                       sino_prec=sino_prec)
        self.__dict__.update(reduced.__dict__)
        self.vecs = v

    def _make_plan(self):
        from .backend import plan_2d_vec

        return plan_2d_vec(self.device, self.vol_prec, self.vol_shape, self.vol_spacing,
                           self.vol_offset, self.sino_prec, self.det_shape, self.vecs)

    def to_vec(self):
        return self.vecs.tolist()


class ConeGeometry:
    """3D flat-panel cone-beam geometry (geometry.py:237-336)."""

    def __init__(self, DSD: float, DSO: float, angles: Union[List[float], List[List[float]]],
                 vol_shape: Tuple[int, int, int], det_shape: Tuple[int, int],
                 det_spacing: Optional[Tuple[float, float]] = None,
                 det_offset: Optional[Tuple[float, float]] = None,
                 det_rotation: Optional[Tuple[float, float, float]] = None,
                 vol_spacing: Optional[Tuple[float, float, float]] = None,
                 vol_offset: Optional[Tuple[float, float, float]] = None,
                 COR: Optional[float] = None, device: int = 0):
        if not is_convertible_to_float(DSD):
            raise TypeError(f"Expected DSD to be float, got {type(DSD)}")
        self.DSD = float(DSD)
        if not is_convertible_to_float(DSO):
            raise TypeError(f"Expected DSO to be float, got {type(DSO)}")
        self.DSO = float(DSO)

        self.det_shape = np.asarray(det_shape)
        if self.det_shape.shape != (2,):
            raise AttributeError(
                f"Detector shape must be two values, got {str(self.det_shape.shape)}")
        self.vol_shape = np.asarray(vol_shape)
        if self.vol_shape.shape != (3,):
            raise AttributeError(
                f"Volume shape must be three values, got {str(self.vol_shape.shape)}")

        self.angles = np.asarray(angles)
        if self.angles.ndim == 1:
            self.nangles = self.angles.shape[0]
            zeros = np.zeros((self.nangles,), dtype=np.float32)
            self.angles = np.vstack((self.angles, zeros, zeros))
        elif self.angles.ndim == 2:
            if self.angles.shape[0] != 3:
                raise AttributeError(
                    "Angles must either be a 1D array, or a 2D array of shape (3, nangles), "
                    f"got {str(self.angles.shape)}")
            self.nangles = self.angles.shape[1]
        else:
            raise AttributeError(
                "Angles must either be a 1D array, or a 2D array of shape (3, nangles), "
                f"got {str(self.angles.shape)}")

        self.det_spacing = self._vec(det_spacing, "det_spacing", 2, np.ones(2))
        self.det_offset = self._vec(det_offset, "det_offset", 2, np.zeros(2))
        self.det_rotation = self._vec(det_rotation, "det_rotation", 3, np.zeros(3))
        if COR is not None:
            if not is_convertible_to_float(COR):
                raise TypeError(f"Expected COR to be float, got {type(COR)}")
            self.COR = float(COR)
        else:
            self.COR = 0.0
        self.vol_spacing = self._vec(vol_spacing, "vol_spacing", 3, np.ones(3))
        self.vol_size = self.vol_shape * self.vol_spacing
        self.vol_offset = self._vec(vol_offset, "vol_offset", 3, np.zeros(3))
        self.device = int(device)
        self._plan = None
        self._exact_plan = None

    @staticmethod
    def _vec(v, name, n, default):
        if v is None:
            return default
        a = np.asarray(v)
        if a.shape != (n,):
            word = {2: "two", 3: "three"}[n]
            raise AttributeError(f"{name} must be {word} values, got {str(a.shape)}")
        return a

    def _make_plan(self):
        from .backend import plan_3d

        return plan_3d(self.device, self.vol_shape, self.vol_spacing, self.vol_offset,
                       self.angles, self.det_shape, self.det_spacing, self.det_offset,
                       self.det_rotation, self.DSO, self.DSD, self.COR)

    @property
    def plan(self):
        """The device plan (``backend.plan_3d``), built on first use."""
        if self._plan is None:
            self._plan = self._make_plan()
        return self._plan

    @property
    def exact_plan(self):
        """A second plan whose forward filters in FP32 (algorithm "quad": the
        same samples and trilinear weights as "registers", 1.8x faster), the
        exact transpose partner of ``adjoint`` (matched gradients)."""
        if self._exact_plan is None:
            self._exact_plan = self._make_plan()
            self._exact_plan.set_algorithm(forward="quad")
        return self._exact_plan

    def sinogram_shape(self):
        return (self.nangles, *self.det_shape)

    def __str__(self):
        return geom_to_str(self)
