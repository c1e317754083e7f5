"""tomosipo's ``tomosipo.astra`` module names, on this package's GPU kernels.

Nothing here uses ASTRA: the module keeps the reference's names so scripts
that import from ``tomosipo.astra`` keep working. ``create_astra_projector``,
``direct_fp`` and ``direct_bp`` are the projector layer
(``tomosipo_gb300.projector``); ``project``/``forward``/``backward`` are the
legacy projection functions on ``Data`` objects (``tomosipo/astra.py:221-371``,
which call ASTRA's ``do_composite``); ``fdk`` reconstructs with FDK
(``tomosipo/astra.py:374-406``, ASTRA's ``accumulate_FDK``).
"""
import torch

from .projector import create_astra_projector, create_projector, direct_bp, direct_fp, direct_project
from . import to_astra, from_astra  # noqa: F401  (tomosipo.astra exports them too)

__all__ = ["create_astra_projector", "direct_fp", "direct_bp", "project", "forward", "backward",
           "fdk", "to_astra", "from_astra"]


def project(*data, voxel_supersampling=1, detector_supersampling=1, forward=None,
            additive=False, projector=None, backprojector="matched"):
    """Project all volume datasets onto all projection datasets, or back.

    As ASTRA's composite projection: forward, every projection dataset becomes
    the sum of the projections of all volume datasets; backward, every volume
    dataset becomes the sum of the backprojections of all projection
    datasets (``additive`` adds to the current values instead). ``projector``
    (from ``create_astra_projector``) is used for every pair; otherwise one is
    built per pair of geometries. ``backprojector`` is ``"matched"`` (the
    exact transpose) or ``"bilinear"`` (ASTRA's voxel-driven kind, which
    honours ``voxel_supersampling``).
    """
    vol_data = [d for d in data if d.is_volume()]
    proj_data = [d for d in data if d.is_projection()]
    if forward is None:
        raise ValueError("project must be given a forward argument (True/False).")
    if len(vol_data) < 1 or len(proj_data) < 1:
        raise ValueError("Expected at least one projection dataset and one volume dataset")
    cache = {}

    def projector_for(vd, pd):
        if projector is not None:
            return projector
        key = (id(vd.geometry), id(pd.geometry))
        if key not in cache:
            cache[key] = create_projector(vd.geometry, pd.geometry,
                                          voxel_supersampling=voxel_supersampling,
                                          detector_supersampling=detector_supersampling)
        return cache[key]

    if forward:
        for pd in proj_data:
            for i, vd in enumerate(vol_data):
                direct_project(projector_for(vd, pd), vd.link, pd.link, forward=True,
                               additive=additive or i > 0)
    else:
        for vd in vol_data:
            for j, pd in enumerate(proj_data):
                direct_project(projector_for(vd, pd), vd.link, pd.link, forward=False,
                               additive=additive or j > 0, bp_kind=backprojector)


def forward(*data, voxel_supersampling=1, detector_supersampling=1, additive=False,
            projector=None):
    """Forward project all volumes onto all projection datasets."""
    project(*data, voxel_supersampling=voxel_supersampling,
            detector_supersampling=detector_supersampling, additive=additive, forward=True,
            projector=projector)


def backward(*data, voxel_supersampling=1, detector_supersampling=1, additive=False,
             projector=None, backprojector="matched"):
    """Backproject all projection datasets onto all volumes."""
    project(*data, voxel_supersampling=voxel_supersampling,
            detector_supersampling=detector_supersampling, additive=additive, forward=False,
            projector=projector, backprojector=backprojector)


def fdk(vol_data, proj_data, *, voxel_supersampling=1, detector_supersampling=1,
        short_scan=False):
    """FDK reconstruction of ``proj_data`` added into ``vol_data``.

    As the reference's ``accumulate_FDK`` call, the reconstruction is added
    to the volume's current values. Any cone-beam geometry
    (``tomosipo_gb300.fdk``); ``short_scan`` adds Parker's redundancy weights
    (not in the reference's call). Supersampling factors are accepted for
    signature compatibility; FDK's backprojection reads the detector once per
    voxel.
    """
    from .fdk import fdk_constants, fdk_reconstruct
    from .projector import _as_device_tensor, _cuda_device_for_host_data

    fdk_constants(vol_data.geometry, proj_data.geometry)  # geometry errors before any device work
    vol, sino = vol_data.data, proj_data.data
    dev = vol.device if isinstance(vol, torch.Tensor) and vol.is_cuda else _cuda_device_for_host_data()
    y, _ = _as_device_tensor(sino, dev, copy_in=True)
    x, copy_back = _as_device_tensor(vol, dev, copy_in=True)
    fdk_reconstruct(vol_data.geometry, proj_data.geometry, y, out=x, additive=True,
                    short_scan=short_scan)
    if copy_back:
        import numpy as np

        target = torch.from_numpy(vol) if isinstance(vol, np.ndarray) else vol
        target.copy_(x)
