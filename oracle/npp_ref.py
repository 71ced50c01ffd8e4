"""The reference's NPP filters on the GPU (TEST INFRASTRUCTURE ONLY).

casm-hella's smoothing (src/hella/src/smooth.cpp:21-127) and SCRUNCH box
filter (src/hella/src/convolution.cu:20-55) run NPP's closed filters, whose
summation order nothing in the reference fixes.  The GPU tests call them
here (oracle/npp/npp_ref.cpp, the _Ctx forms) to measure this library's
own filter arithmetic against what the reference actually computes.  Only
tests load this module; the product never links NPP.
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "build" / "libnpp_ref.so"
_lib = None
_VP = C.c_void_p


def build() -> Path:
    r = subprocess.run(["make", "-s", "-C", str(HERE), "npp"], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"NPP shim build failed\n{r.stdout}\n{r.stderr}")
    return LIB_PATH


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(str(LIB_PATH))
        for n in ("nr_filter_f32", "nr_filter_f16"):
            f = getattr(L, n)
            f.restype = C.c_int
            f.argtypes = [_VP, C.c_int, C.c_int, C.c_int, _VP, C.c_int, _VP, C.c_int, C.c_int, C.c_int, C.c_int,
                          _VP]
        _lib = L
    return _lib


def smooth_planes(dd: np.ndarray, taps3: list[np.ndarray], wmax: int, ntime_out: int) -> np.ndarray:
    """smooth.cpp:42-84 with NPP: for each 3 x (2sm+1) kernel in taps3, the
    filter over the whole [ndms][ntime_dd] plane (anchor {0,1}, replicate
    border), then the crop of rows 1..ndms-2 and columns wmax/2 ..
    wmax/2 + ntime_out.  Returns the pre-normalisation planes
    [nbox][ndms-2][ntime_out]."""
    import torch

    L = lib()
    dd = np.ascontiguousarray(dd, np.float32)
    ndms, ntd = dd.shape
    d_in = torch.from_numpy(dd).cuda()
    d_out = torch.empty_like(d_in)
    stream = torch.cuda.current_stream().cuda_stream
    out = np.zeros((len(taps3), ndms - 2, ntime_out), np.float32)
    for b, k in enumerate(taps3):
        k = np.ascontiguousarray(k, np.float32)
        d_k = torch.from_numpy(k.reshape(-1)).cuda()
        rc = L.nr_filter_f32(d_in.data_ptr(), ntd * 4, ntd, ndms, d_out.data_ptr(), ntd * 4, d_k.data_ptr(),
                             k.shape[1], k.shape[0], 0, 1, stream)
        assert rc == 0, f"nppiFilterBorder_32f_C1R_Ctx returned {rc}"
        torch.cuda.synchronize()
        full = d_out.cpu().numpy()
        out[b] = full[1:ndms - 1, wmax // 2: wmax // 2 + ntime_out]
    return out


def box_filter_f16(plane: np.ndarray, xw: int, yw: int, scfac: float) -> np.ndarray:
    """convolution.cu:20-55 with NPP: an xw x yw kernel of scfac (float),
    anchor {xw/2, yw/2}, replicate border, over an fp16 plane given as uint16
    bit patterns [height][stride] (the whole stride, as the reference)."""
    import torch

    L = lib()
    plane = np.ascontiguousarray(plane, np.uint16)
    h, w = plane.shape
    d_in = torch.from_numpy(plane.view(np.int16)).cuda()
    d_out = torch.empty_like(d_in)
    d_k = torch.full((xw * yw,), float(np.float32(scfac)), dtype=torch.float32, device="cuda")
    rc = L.nr_filter_f16(d_in.data_ptr(), w * 2, w, h, d_out.data_ptr(), w * 2, d_k.data_ptr(), xw, yw, xw // 2,
                         yw // 2, torch.cuda.current_stream().cuda_stream)
    assert rc == 0, f"nppiFilterBorder32f_16f_C1R_Ctx returned {rc}"
    torch.cuda.synchronize()
    return d_out.cpu().numpy().view(np.uint16)
