"""Runs the reference's own CUDA kernel, as a measured baseline on the same GPU.

Test and measurement infrastructure, not product code: only the tests and the benchmark's
baseline legs use it.  ``oracle/ref_gpu_build.py`` compiles ``simus_fused_kernel`` from the
reference's ``src/fast_simus/kernels/simus_fused.cu`` into ``oracle/_ref/*.fatbin``; this module
loads that binary with the CUDA driver API (``cuModuleLoadData`` / ``cuLaunchKernel`` through
ctypes, on PyTorch's primary context and current stream) and feeds it the inputs that the
reference's ``simus_cuda`` wrapper would, restated here in PyTorch:

* ``_prepare_inputs`` (kernels/cuda_simus.py:109-226): float32 scatterer x/z padded to a
  multiple of B_SCAT with the first scatterer and rc = 0, float32 element centres, angles and
  sub-element offsets, ``apod * exp(i 2 pi f0 tau)`` and ``2 pi df tau`` per element,
  pulse*probe as complex64, probe as float32, and the 10 float scalars;
* ``simus_cuda`` (kernels/cuda_simus.py:232-321): zeroed float32 ``spect_re/spect_im``
  ``(E, F)``, ``GRID_BLOCKS`` x ``TG_SIZE`` launch with the kernel's dynamic shared memory, and
  the ``(F, E)`` complex64 result (the selected band before the correction factor).
"""

from __future__ import annotations

import ctypes
import json
import math
from pathlib import Path

import numpy as np
import torch

from oracle import fastsimus_fp64 as O

REF_DIR = Path(__file__).resolve().parent / "_ref"
_MANIFEST = REF_DIR / "ref_kernels.json"
_CU_FUNC_ATTRIBUTE_MAX_DYNAMIC_SHARED_SIZE_BYTES = 8

_drv = None


def _driver():
    global _drv
    if _drv is None:
        lib = ctypes.CDLL("libcuda.so.1")
        P = ctypes.POINTER
        for name, args in (("cuInit", [ctypes.c_uint]),
                           ("cuCtxGetCurrent", [P(ctypes.c_void_p)]),
                           ("cuModuleLoadData", [P(ctypes.c_void_p), ctypes.c_void_p]),
                           ("cuModuleGetFunction", [P(ctypes.c_void_p), ctypes.c_void_p, ctypes.c_char_p]),
                           ("cuModuleUnload", [ctypes.c_void_p]),
                           ("cuFuncSetAttribute", [ctypes.c_void_p, ctypes.c_int, ctypes.c_int]),
                           ("cuLaunchKernel", [ctypes.c_void_p] + [ctypes.c_uint] * 7 +
                            [ctypes.c_void_p, P(ctypes.c_void_p), P(ctypes.c_void_p)]),
                           ("cuGetErrorString", [ctypes.c_int, P(ctypes.c_char_p)])):
            fn = getattr(lib, name)
            fn.argtypes = args
            fn.restype = ctypes.c_int
        _drv = lib
    return _drv


def _check(rc: int, what: str):
    if rc != 0:
        msg = ctypes.c_char_p()
        _driver().cuGetErrorString(rc, ctypes.byref(msg))
        raise RuntimeError(f"{what} failed: CUDA driver error {rc} ({(msg.value or b'').decode()})")


def available(E: int | None = None, U: int | None = None, F: int | None = None) -> tuple[bool, str]:
    """Whether the prebuilt reference kernel exists (for this shape, when given)."""
    if not _MANIFEST.is_file():
        return False, "oracle/_ref/ref_kernels.json absent (oracle/ref_gpu_build.py not run)"
    if E is not None:
        key = f"E{E}_U{U}_F{F}"
        m = json.loads(_MANIFEST.read_text())
        if key not in m or not (REF_DIR / m[key]["file"]).is_file():
            return False, f"no reference kernel built for shape {key}"
    return True, ""


class RefSimusKernel:
    """The reference's ``simus_fused_kernel`` for one compile-time shape (E, U, F)."""

    def __init__(self, n_elements: int, n_sub: int, n_freq: int, device: torch.device | None = None):
        ok, why = available(n_elements, n_sub, n_freq)
        if not ok:
            raise FileNotFoundError(why)
        info = json.loads(_MANIFEST.read_text())[f"E{n_elements}_U{n_sub}_F{n_freq}"]
        self.E, self.U, self.F = n_elements, n_sub, n_freq
        self.defines = info["defines"]
        self.b_scat = int(self.defines["B_SCAT"])
        self.grid, self.block, self.shmem = int(info["grid_blocks"]), int(info["block_threads"]), int(info["shmem_bytes"])
        self.device = torch.device(device or "cuda")
        if self.device.index is None:
            self.device = torch.device("cuda", torch.cuda.current_device())
        torch.cuda.set_device(self.device)
        torch.zeros(1, device=self.device)  # primary context current on this thread
        drv = _driver()
        _check(drv.cuInit(0), "cuInit")
        ctx = ctypes.c_void_p()
        _check(drv.cuCtxGetCurrent(ctypes.byref(ctx)), "cuCtxGetCurrent")
        if not ctx.value:
            raise RuntimeError("no current CUDA context")
        self._image = ctypes.create_string_buffer((REF_DIR / info["file"]).read_bytes())
        self._mod = ctypes.c_void_p()
        _check(drv.cuModuleLoadData(ctypes.byref(self._mod), ctypes.cast(self._image, ctypes.c_void_p)),
               "cuModuleLoadData")
        self._fn = ctypes.c_void_p()
        _check(drv.cuModuleGetFunction(ctypes.byref(self._fn), self._mod, b"simus_fused_kernel"),
               "cuModuleGetFunction")
        if self.shmem > 48 * 1024:
            _check(drv.cuFuncSetAttribute(self._fn, _CU_FUNC_ATTRIBUTE_MAX_DYNAMIC_SHARED_SIZE_BYTES, self.shmem),
                   "cuFuncSetAttribute")

    # ---- kernels/cuda_simus.py:109-226 -------------------------------------------------------
    def prepare(self, scatterers, rc, delays, plan, params, medium, tx_apodization=None) -> dict:
        dev = self.device
        f32 = dict(dtype=torch.float32, device=dev)
        c, alpha = medium.speed_of_sound, medium.attenuation
        E, U = params.n_elements, int(plan.n_sub)
        F = int(plan.selected_freqs.shape[0])
        if (E, U, F) != (self.E, self.U, self.F):
            raise ValueError(f"kernel compiled for {(self.E, self.U, self.F)}, inputs give {(E, U, F)}")
        dclean, apod = O._clean(delays, tx_apodization, E)
        epos, theta, apex = O.element_positions(E, params.pitch, params.radius)
        theta = np.zeros(E, dtype=np.float32) if theta is None else theta
        offs = O.subelement_centroids(params.element_width, U, np.asarray(theta, dtype=np.float64))
        fsel = np.asarray(plan.selected_freqs, dtype=np.float64)
        f0 = float(fsel[0])
        df = float(fsel[1] - fsel[0]) if F > 1 else 0.0
        pp = (np.asarray(plan.pulse_spectrum) * np.asarray(plan.probe_spectrum)).astype(np.complex64)
        scat = np.asarray(scatterers, dtype=np.float64).reshape(-1, 2)
        rcv = np.asarray(rc, dtype=np.float64).reshape(-1)
        n = scat.shape[0]
        n_pad = ((n + self.b_scat - 1) // self.b_scat) * self.b_scat
        sx = np.concatenate([scat[:, 0], np.repeat(scat[:1, 0], n_pad - n)]).astype(np.float32)
        sz = np.concatenate([scat[:, 1], np.repeat(scat[:1, 1], n_pad - n)]).astype(np.float32)
        rcp = np.concatenate([rcv, np.zeros(n_pad - n)]).astype(np.float32)
        t = lambda a: torch.as_tensor(np.ascontiguousarray(a, dtype=np.float32), **f32)  # noqa: E731
        return {
            "scat_x": t(sx), "scat_z": t(sz), "rc": t(rcp),
            "elem_x": t(epos[:, 0]), "elem_z": t(epos[:, 1]),
            "cos_te": t(np.cos(theta)), "sin_neg_te": t(np.sin(-np.asarray(theta))),
            "sub_dx": t(offs[..., 0].reshape(-1)), "sub_dz": t(offs[..., 1].reshape(-1)),
            "da_init_re": t(np.cos(2 * math.pi * f0 * dclean) * apod),
            "da_init_im": t(np.sin(2 * math.pi * f0 * dclean) * apod),
            "dps": t(2 * math.pi * df * dclean),
            "pp_re": t(pp.real), "pp_im": t(pp.imag), "probe_real": t(plan.probe_spectrum),
            "n_scat": n_pad,
            "scalars": [2 * math.pi * f0 / c, alpha / O.NEPER_TO_DB * f0 / 1e6 * 1e2,
                        2 * math.pi * df / c, alpha / O.NEPER_TO_DB * df / 1e6 * 1e2,
                        c / params.freq_center / 2.0, float(plan.seg_length),
                        2 * math.pi * params.freq_center / c, 1.0 / U,
                        1e31 if params.radius == math.inf else float(params.radius), float(apex)],
        }

    # ---- kernels/cuda_simus.py:273-321 -------------------------------------------------------
    def launch(self, d: dict, spect_re: torch.Tensor, spect_im: torch.Tensor, stream=None) -> None:
        """Zero the (E, F) outputs and launch on `stream` (default: PyTorch's current stream)."""
        spect_re.zero_()
        spect_im.zero_()
        ptr_names = ("scat_x", "scat_z", "rc", "elem_x", "elem_z", "cos_te", "sin_neg_te", "sub_dx", "sub_dz",
                     "da_init_re", "da_init_im", "dps", "pp_re", "pp_im", "probe_real")
        vals = [ctypes.c_void_p(d[k].data_ptr()) for k in ptr_names]
        vals += [ctypes.c_void_p(spect_re.data_ptr()), ctypes.c_void_p(spect_im.data_ptr()),
                 ctypes.c_int32(d["n_scat"])]
        vals += [ctypes.c_float(v) for v in d["scalars"]]
        params = (ctypes.c_void_p * len(vals))(*[ctypes.cast(ctypes.pointer(v), ctypes.c_void_p) for v in vals])
        s = stream if stream is not None else torch.cuda.current_stream(self.device)
        _check(_driver().cuLaunchKernel(self._fn, self.grid, 1, 1, self.block, 1, 1, self.shmem,
                                        ctypes.c_void_p(s.cuda_stream), params, None), "cuLaunchKernel")

    def outputs(self):
        return (torch.empty(self.E * self.F, dtype=torch.float32, device=self.device),
                torch.empty(self.E * self.F, dtype=torch.float32, device=self.device))

    def spectrum(self, scatterers, rc, delays, plan, params, medium, tx_apodization=None) -> torch.Tensor:
        """(F, E) complex64 selected-band spectrum, as ``simus_cuda`` returns it."""
        d = self.prepare(scatterers, rc, delays, plan, params, medium, tx_apodization)
        re, im = self.outputs()
        self.launch(d, re, im)
        torch.cuda.current_stream(self.device).synchronize()
        return torch.complex(re, im).reshape(self.E, self.F).T.contiguous()

    def close(self):
        if self._mod.value:
            _driver().cuModuleUnload(self._mod)
            self._mod = ctypes.c_void_p()
