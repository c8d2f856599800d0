"""Projection of exit directions onto the EBSD detector on the GPU.

projOnDetector keeps the reference's signature and meaning
(MC/tools/rotation.py:78-102): each escape direction is rotated by the
conjugate of q_SD = (cos(alpha/2), sin(alpha/2), 0, 0), the translation
(x_PC, y_PC, L) is subtracted and the x, y components are returned.  The
work runs in the mcd_project_detector kernel; project() is the device-array
form used on transport output without leaving the GPU.

The default geometry is the reference's (MC/tools/parameters.py:22-33):
L = 15250 um, sample tilt 70 deg, theta_C = 0, alpha = 90 - 70 + 0 deg,
pixel pitch 49.375 um, pattern centre (3.57, 113.45) pixels.
"""
import numpy as np

from . import _lib
from .engine import _torch

L = 15250.0
SIGMA = 70.0
THETA_C = 0.0
ALPHA = 90.0 - SIGMA + THETA_C
DELTA = 49.375
X_PIXELS, Y_PIXELS = 640, 480
X_PC, Y_PC = 3.57, 113.45
XY_PC = (X_PC * DELTA, Y_PC * DELTA)


def project(dirs, alpha=ALPHA, xy_PC=XY_PC, L=L, out=None, stream=None):
    """dirs: CUDA tensor (3, n) of float32 or float64 direction planes (the
    layout of the transport's per-electron 'dir' output).  Returns (2, n)."""
    torch = _torch()
    if not dirs.is_cuda or dirs.dim() != 2 or dirs.shape[0] != 3:
        raise ValueError("dirs must be a CUDA tensor of shape (3, n)")
    if dirs.dtype not in (torch.float32, torch.float64):
        raise TypeError("dirs must be float32 or float64")
    dirs = dirs.contiguous()
    n = dirs.shape[1]
    if out is None:
        out = torch.empty((2, n), dtype=dirs.dtype, device=dirs.device)
    elif out.shape != (2, n) or out.dtype != dirs.dtype or not out.is_contiguous():
        raise ValueError("out must be a contiguous (2, n) tensor of the dirs dtype")
    st = stream if stream is not None else torch.cuda.current_stream(dirs.device)
    prec = _lib.FP32 if dirs.dtype == torch.float32 else _lib.FP64
    code = _lib.lib().mcd_project_detector(dirs.data_ptr(), n, prec, float(alpha), float(xy_PC[0]),
                                           float(xy_PC[1]), float(L), out.data_ptr(), st.cuda_stream)
    _lib.check("mcd_project_detector", code)
    return out


def projOnDetector(xyz_exit, alpha, xy_PC, L):
    """MC/tools/rotation.py:78-102: list of escape direction vectors -> list
    of (x, y) arrays on the detector, computed in FP64 on the GPU."""
    torch = _torch()
    v = np.asarray([np.asarray(d, dtype=np.float64) for d in xyz_exit], dtype=np.float64).reshape(-1, 3)
    dev = torch.device("cuda")
    planes = torch.from_numpy(np.ascontiguousarray(v.T)).to(dev)
    xy = project(planes, alpha, xy_PC, L).cpu().numpy()
    return [xy[:, i].copy() for i in range(v.shape[0])]
