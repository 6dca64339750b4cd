"""Drop-in for the wire <-> grid pieces of rhoPJ.py used by the 3-D coupling
(CalcJfx :491, QWPlacement :655) on the GPU.  numpy inputs are copied to the
device and results come back as numpy; CUDA tensors stay on the device."""

import numpy as np
import torch

from . import _lib
from .wires import CDTYPE


def _dev(x, dtype):
    if isinstance(x, torch.Tensor):
        return (x if x.is_cuda else x.cuda()).to(dtype).contiguous(), True
    return torch.from_numpy(np.ascontiguousarray(np.asarray(x))).to("cuda", dtype).contiguous(), False


def CalcJfx(RhoNew, RhoPrev, dt, dx):
    """rhoPJ.py:491-515: free current from the charge change, J_i = J_{i-1} - drho_i/dt dx."""
    rn, was = _dev(RhoNew, CDTYPE)
    rp, _ = _dev(RhoPrev, CDTYPE)
    J = torch.empty_like(rn)
    _lib.check(_lib.load().sbe_calc_jfx(rn.numel(), _lib.ptr(rn), _lib.ptr(rp), float(dt),
                                        float(dx), _lib.ptr(J), _lib.stream_handle()), "CalcJfx")
    return J if was else J.cpu().numpy()


def QWPlacement(Fwire, gx, gy, gz, Fgrid):
    """rhoPJ.py:655-702: Fgrid[i, j, k] = gx[i] gy[j] gz[k] Fwire[i], in place."""
    fw, _ = _dev(Fwire, CDTYPE)
    g = [_dev(np.real(a) if not isinstance(a, torch.Tensor) else a.real, torch.float64)[0]
         for a in (gx, gy, gz)]
    nx, ny, nz = Fgrid.shape
    out = Fgrid if isinstance(Fgrid, torch.Tensor) and Fgrid.is_cuda and Fgrid.is_contiguous() \
        and Fgrid.dtype == CDTYPE else torch.empty((nx, ny, nz), dtype=CDTYPE, device="cuda")
    _lib.check(_lib.load().sbe_qw_placement(nx, ny, nz, _lib.ptr(fw), *[_lib.ptr(a) for a in g],
                                            _lib.ptr(out), _lib.stream_handle()), "QWPlacement")
    if out is not Fgrid:
        if isinstance(Fgrid, torch.Tensor):
            Fgrid.copy_(out)
        else:
            Fgrid[...] = out.cpu().numpy()
