"""Drop-in for the wire <-> grid pieces of rhoPJ.py used by the 3-D coupling
(CalcJfx :491, QWPlacement :655, ElongfromRho :703) on the GPU.  numpy inputs are
copied to the device and results come back as numpy; CUDA tensors stay on the
device."""

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


_grids = {}


def ElongfromRho(space, Rho, Px, Py, Pz, ExlfromPRho, EylfromPRho, EzlfromPRho, ExlfromP,
                 EylfromP, EzlfromP, ExlfromRho, EylfromRho, EzlfromRho, RhoBound):
    """rhoPJ.py:703-880: longitudinal fields from the charge Rho and the polarisation
    (Px, Py, Pz) in k space, with the space's own wavenumber tables (GetKxArray,
    GetKyArray, GetKzArray, typespace.py:958-1030) and epsr (GetEpsr); all ten outputs
    filled in place, and Px, Py, Pz replaced by their transforms as the reference does.
    ``space`` is any object with Nx, Ny, Nz, dx, dy, dz, epsr (the typespace ss fields)
    and the k tables are the reference's centred arrays."""
    from .pstd import Pstd3D
    n = (int(space.Nx), int(space.Ny), int(space.Nz))
    d = (float(space.dx), float(space.dy), float(space.dz))
    epsr = 1.0 if n[2] == 1 else float(space.epsr)     # GetEpsr, typespace.py:536-560
    key = (n, d, epsr)
    if key not in _grids:
        _grids[key] = Pstd3D(n, d, epsr)
    g = _grids[key]
    # GetKxArray = GetKArray(Nx, GetXWidth) with GetXWidth = dx (Nx - 1)
    q = [_centred_k(nn, dd * (nn - 1)) for nn, dd in zip(n, d)]
    rho, _ = _dev(Rho, CDTYPE)
    P = torch.stack([_dev(a, CDTYPE)[0].reshape(n) for a in (Px, Py, Pz)])
    out, pk = g.elong(rho.reshape(n), P, *q)
    targets = (ExlfromPRho, EylfromPRho, EzlfromPRho, ExlfromP, EylfromP, EzlfromP, ExlfromRho,
               EylfromRho, EzlfromRho, RhoBound)
    for t, v in zip(targets, out):
        _put(t, v)
    for t, v in zip((Px, Py, Pz), pk):
        _put(t, v)


def _centred_k(n, L):
    """typespace.py:852-910 GetKArray: n values spaced 2 pi / L, centred at index n // 2."""
    if n == 1:
        return np.zeros(1)
    k = np.arange(n, dtype=float) * (2.0 * np.pi / L if L > 0 else 1.0)
    return k - k[n // 2]


def _put(target, v):
    if isinstance(target, torch.Tensor):
        target.copy_(v.reshape(target.shape))
    else:
        target[...] = v.reshape(target.shape).cpu().numpy()
