"""Drop-in for the grid sampling of usefulsubs.py used by the 3-D coupling (EAtXYZ
:1996 with locator :1803) on the GPU, plus a batched form over many points."""

import numpy as np
import torch

from . import _lib
from .rhoPJ import _dev
from .wires import CDTYPE


def EAtXYZ_points(f, x, y, z, pts):
    """Trilinear samples of f (nx, ny, nz) at pts (npts, 3): EAtXYZ for every point."""
    ft, was = _dev(f, CDTYPE)
    ax = [_dev(a, torch.float64)[0] for a in (x, y, z)]
    p, _ = _dev(pts, torch.float64)
    n = p.numel() // 3
    out = torch.empty(n, dtype=CDTYPE, device="cuda")
    _lib.check(_lib.load().sbe_e_at_xyz(_lib.ptr(ft), _lib.ptr(ax[0]), ax[0].numel(),
                                        _lib.ptr(ax[1]), ax[1].numel(), _lib.ptr(ax[2]),
                                        ax[2].numel(), _lib.ptr(p), n, _lib.ptr(out),
                                        _lib.stream_handle()), "EAtXYZ")
    return out if was else out.cpu().numpy()


def EAtXYZ(f, x, y, z, x0, y0, z0):
    """usefulsubs.py:1996-2075: the trilinear sample of f at (x0, y0, z0)."""
    return complex(EAtXYZ_points(f, x, y, z, np.array([[x0, y0, z0]], dtype=float))[0])
