"""Tomographic operator ``A = ts.operator(vg, pg)`` (``tomosipo/Operator.py``).

Same API as tomosipo: ``A(x, out=None)``, ``A.T(y, out=None)``, ``A.T.T is A``,
``domain``/``range``, ``domain_shape``/``range_shape``, ``additive``. A
``VolumeVectorGeometry`` is first moved, together with the projection
geometry, into a frame where the volume is axis-aligned at the origin
(``tomosipo/Operator.py:11-60``).

One addition: ``backprojector`` selects the backprojection. ``"matched"``
(default) is the exact transpose of the forward projector, so ``A.T`` is the
adjoint of ``A`` to fp32 rounding (what gradients and SIRT convergence rely
on). ``"bilinear"`` is ASTRA's style of backprojector: voxel-driven with
bilinear detector interpolation, an approximation of the adjoint.
"""
import numpy as np

from . import vector_calc as vc
from .geometry import VolumeGeometry, VolumeVectorGeometry, volume, from_perspective
from .Data import Data, data
from .links.base import link, geometry_shape
from .projector import create_projector, direct_fp, direct_bp, direct_project_batch, BP_KINDS


def to_astra_compatible_operator_geometry(vg, pg):
    """Axis-aligned volume at the origin and the projection geometry moved with it."""
    if isinstance(vg, VolumeGeometry):
        return vg, pg
    if not isinstance(vg, VolumeVectorGeometry):
        raise TypeError(f"Expected volume geometry. Got {type(vg)}. ")
    vg = vg.to_vec()
    P = from_perspective(
        pos=vg.pos,
        w=vg.w / vc.norm(vg.w)[:, None],
        v=vg.v / vc.norm(vg.v)[:, None],
        u=vg.u / vc.norm(vg.u)[:, None],
    )
    vg2 = P * vg
    pg2 = P * pg.to_vec()
    vs = vg2.voxel_size
    if not (
        np.allclose(vg2.pos, 0)
        and np.allclose(vg2.w, vs[0] * np.array([1, 0, 0]))
        and np.allclose(vg2.v, vs[1] * np.array([0, 1, 0]))
        and np.allclose(vg2.u, vs[2] * np.array([0, 0, 1]))
    ):
        raise ValueError("Volume vector geometry could not be made axis-aligned (skewed axes?).")
    return volume(shape=vg2.shape, pos=0, size=vg2.size), pg2


def operator(volume_geometry, projection_geometry, voxel_supersampling=1,
             detector_supersampling=1, additive=False, backprojector="matched"):
    """Create a new tomographic operator (``tomosipo/Operator.py:63-106``).

    ``detector_supersampling`` d: the forward projection averages d x d rays
    per detector pixel, and the matched backprojection is its exact
    transpose. ``voxel_supersampling`` d: the bilinear backprojection
    (``backprojector="bilinear"``, ASTRA's voxel-driven kind) averages d^3
    points per voxel. The matched backprojection (the default) is the exact
    transpose of the forward projection, which samples rays and not voxels,
    so voxel supersampling does not change it.
    """
    return Operator(
        volume_geometry,
        projection_geometry,
        voxel_supersampling=voxel_supersampling,
        detector_supersampling=detector_supersampling,
        additive=additive,
        backprojector=backprojector,
    )


def _to_link(geometry, x):
    """A dataset's own link, or a new link around an array
    (``tomosipo/Operator.py:109-113``)."""
    if isinstance(x, Data):
        return x.link
    return link(geometry, x)


class Operator:
    """A linear tomographic projection operator."""

    def __init__(self, volume_geometry, projection_geometry, voxel_supersampling=1,
                 detector_supersampling=1, additive=False, backprojector="matched"):
        if backprojector not in BP_KINDS:
            raise ValueError(
                f"backprojector must be one of {sorted(BP_KINDS)}. Got {backprojector!r}."
            )
        self.volume_geometry = volume_geometry
        self.projection_geometry = projection_geometry
        vg, pg = to_astra_compatible_operator_geometry(volume_geometry, projection_geometry)
        self.astra_compat_vg = vg
        self.astra_compat_pg = pg
        self.projector = create_projector(
            vg, pg, voxel_supersampling=voxel_supersampling,
            detector_supersampling=detector_supersampling,
        )
        self.astra_projector = self.projector  # tomosipo attribute name
        self.voxel_supersampling = voxel_supersampling
        self.detector_supersampling = detector_supersampling
        self.additive = additive
        self.backprojector = backprojector
        self._transpose = BackprojectionOperator(self)

    def _fp(self, volume, out=None):
        vlink = _to_link(self.astra_compat_vg, volume)
        if out is not None:
            plink = _to_link(self.astra_compat_pg, out)
        elif self.additive:
            plink = vlink.new_zeros(self.range_shape)
        else:
            plink = vlink.new_empty(self.range_shape)
        direct_fp(self.projector, vlink, plink, additive=self.additive)
        if isinstance(volume, Data):  # a dataset in, a dataset out (tomosipo/Operator.py:189-192)
            return data(self.projection_geometry, plink.data)
        return plink.data

    def _bp(self, projection, out=None):
        plink = _to_link(self.astra_compat_pg, projection)
        if out is not None:
            vlink = _to_link(self.astra_compat_vg, out)
        elif self.additive:
            vlink = plink.new_zeros(self.domain_shape)
        else:
            vlink = plink.new_empty(self.domain_shape)
        direct_bp(self.projector, vlink, plink, additive=self.additive,
                  bp_kind=self.backprojector)
        if isinstance(projection, Data):  # tomosipo/Operator.py:230-233
            return data(self.volume_geometry, vlink.data)
        return vlink.data

    def __call__(self, volume, out=None):
        """Forward project ``volume``; writes into ``out`` when given."""
        return self._fp(volume, out)

    def _apply_batch(self, volumes, out):
        """out[i] = A(volumes[i]) (or += when additive) for stacked CUDA float32
        tensors (n, z, y, x) -> (n, rows, angles, cols), in one C-ABI call."""
        direct_project_batch(self.projector, volumes, out, forward=True, additive=self.additive)

    def _bp_batch(self, projections, out):
        direct_project_batch(self.projector, out, projections, forward=False,
                             additive=self.additive, bp_kind=self.backprojector)

    def transpose(self):
        return self._transpose

    @property
    def T(self):
        return self.transpose()

    @property
    def domain(self):
        return self.volume_geometry

    @property
    def range(self):
        return self.projection_geometry

    @property
    def domain_shape(self):
        return geometry_shape(self.astra_compat_vg)

    @property
    def range_shape(self):
        return geometry_shape(self.astra_compat_pg)


class BackprojectionOperator:
    """Transpose of an operator; ``A.T is A.T.T.T``."""

    def __init__(self, parent):
        self.parent = parent

    def __call__(self, projection, out=None):
        return self.parent._bp(projection, out)

    def _apply_batch(self, projections, out):
        """out[i] = A.T(projections[i]) for stacked CUDA float32 tensors, in one C-ABI call."""
        self.parent._bp_batch(projections, out)

    def transpose(self):
        return self.parent

    @property
    def T(self):
        return self.transpose()

    @property
    def domain(self):
        return self.parent.range

    @property
    def range(self):
        return self.parent.domain

    @property
    def domain_shape(self):
        return self.parent.range_shape

    @property
    def range_shape(self):
        return self.parent.domain_shape
