"""Test phantoms (``tomosipo/phantom.py``)."""
import numpy as np


def hollow_box(vd):
    """Fill a volume array (or ``.data`` holder) with a hollow box phantom.

    The box spans 20%..80% of each axis and its 40%..60% core is empty
    (``tomosipo/phantom.py:4-25``). Works on NumPy arrays and torch tensors
    in place and returns its argument.
    """
    data = vd.data if hasattr(vd, "data") and not isinstance(vd, np.ndarray) and not _is_tensor(vd) else vd
    shape = np.array(data.shape)
    s20 = shape * 20 // 100
    s40 = shape * 40 // 100
    data[...] = 0.0
    data[tuple(slice(a, n - a) for a, n in zip(s20, shape))] = 1.0
    data[tuple(slice(a, n - a) for a, n in zip(s40, shape))] = 0.0
    return vd


def _is_tensor(x):
    try:
        import torch

        return isinstance(x, torch.Tensor)
    except ImportError:
        return False
