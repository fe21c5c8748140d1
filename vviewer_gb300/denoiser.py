"""Learned denoiser (vvpt_denoiser_*): a U-Net over noisy radiance, albedo and
normal, trained on the GPU by the library's own BF16 tensor-core kernels.
Images are torch CUDA tensors [n, h, w, 4] float32 (RGBA)."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native as N


class Denoiser:
    def __init__(self, ctx, seed: int = 1):
        self.ctx = ctx
        h = C.c_void_p()
        ctx.check(ctx.lib.vvpt_denoiser_create(ctx.handle, int(seed), C.byref(h)))
        self.handle = h
        n = C.c_uint64()
        ctx.check(ctx.lib.vvpt_denoiser_num_params(self.handle, C.byref(n)))
        self.num_params = int(n.value)

    def close(self) -> None:
        if self.handle:
            self.ctx.lib.vvpt_denoiser_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    KERNELS = {"tcgen05": 0, "mma_sync": 1, "tcgen05_tiles": 2, "tcgen05_persistent": 3, "tcgen05_unfused": 4,
               "tcgen05_wgrad": 5}

    def set_kernels(self, kind: str) -> None:
        """Convolution kernels: 'tcgen05' (default: strip kernel where the
        weights fit in shared memory, per-tile kernels elsewhere),
        'mma_sync', 'tcgen05_tiles' (per-tile tcgen05 kernels only),
        'tcgen05_persistent' (strip kernel on a 16-CTA grid),
        'tcgen05_unfused' (inference writes the upsample + concat tensor) or
        'tcgen05_wgrad' (weight gradients on tcgen05 as well)."""
        self.ctx.check(self.ctx.lib.vvpt_denoiser_set_kernels(self.handle, self.KERNELS[kind]))

    def inject_wait_timeout(self) -> None:
        """Diagnostics: the next strip convolution's bounded waits run out
        (vvpt_denoiser_inject_wait_timeout); the next call reports it."""
        self.ctx.check(self.ctx.lib.vvpt_denoiser_inject_wait_timeout(self.handle))

    def params(self) -> np.ndarray:
        out = np.zeros(self.num_params, dtype=np.float32)
        self.ctx.check(self.ctx.lib.vvpt_denoiser_get_params(self.handle, out.ctypes.data, self.num_params))
        return out

    def set_params(self, p: np.ndarray) -> None:
        p = np.ascontiguousarray(p, dtype=np.float32)
        assert p.size == self.num_params
        self.ctx.check(self.ctx.lib.vvpt_denoiser_set_params(self.handle, p.ctypes.data, self.num_params))

    @staticmethod
    def _batch(radiance, albedo, normal, target) -> N.DenoiseBatch:
        n, h, w, c = radiance.shape
        for t in (radiance, albedo, normal, target):
            assert t.is_cuda and t.is_contiguous() and tuple(t.shape) == (n, h, w, 4)
        return N.DenoiseBatch(radiance.data_ptr(), albedo.data_ptr(), normal.data_ptr(), target.data_ptr(), n, w, h)

    def gradients(self, radiance, albedo, normal, target) -> tuple[float, np.ndarray]:
        b = self._batch(radiance, albedo, normal, target)
        g = np.zeros(self.num_params, dtype=np.float32)
        loss = C.c_float()
        self.ctx.check(self.ctx.lib.vvpt_denoiser_gradients(self.handle, C.byref(b), g.ctypes.data, self.num_params,
                                                            C.byref(loss)))
        return float(loss.value), g

    def train_step(self, radiance, albedo, normal, target, lr: float = 1e-3) -> float:
        b = self._batch(radiance, albedo, normal, target)
        loss = C.c_float()
        self.ctx.check(self.ctx.lib.vvpt_denoiser_train_step(self.handle, C.byref(b), float(lr), C.byref(loss)))
        return float(loss.value)

    def apply(self, radiance, albedo, normal, out) -> None:
        """One image: [h, w, 4] CUDA tensors in, out [h, w, 4] written."""
        h, w, _ = radiance.shape
        self.ctx.check(self.ctx.lib.vvpt_denoiser_apply(self.handle, radiance.data_ptr(), albedo.data_ptr(),
                                                        normal.data_ptr(), out.data_ptr(), w, h))

    def save(self, path) -> None:
        """Writes the network's parameters (float32) to an .npz file."""
        np.savez_compressed(path, params=self.params())

    def load(self, path) -> None:
        """Reads parameters written by save()."""
        with np.load(path) as z:
            self.set_params(z["params"])


class DenoiserStep:
    """The denoising step of the output stage (the OIDN call of
    VulkanRendererPathTracing.cpp:985-1018) over host images: radiance,
    albedo and normal as the renderer returns them (H x W x 4 float32; the
    normal buffer stored as n * 0.5 + 0.5, the form the network is trained
    on). Returns the denoised radiance, alpha 1."""

    def __init__(self, denoiser: Denoiser):
        self.denoiser = denoiser

    def denoise(self, radiance: np.ndarray, albedo: np.ndarray, normal: np.ndarray) -> np.ndarray:
        import torch

        bufs = [torch.from_numpy(np.ascontiguousarray(x, dtype=np.float32)).cuda() for x in (radiance, albedo, normal)]
        out = torch.zeros_like(bufs[0])
        self.denoiser.apply(*bufs, out)
        torch.cuda.synchronize()
        return out.cpu().numpy()
