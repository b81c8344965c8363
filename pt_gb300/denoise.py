"""Learned denoiser: Python mirror of include/pt_denoise.h.

`UNet` owns a native network (pt_unet_*) for a fixed batch and image size;
parameters move as flat float32 numpy arrays in the library's order (per
layer w[9][c_in][c_out], then b[c_out]).  Device buffers handed to the
network are plain device addresses (torch tensors serve as the allocator in
the training and benchmark scripts).
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from . import abi

WEIGHTS_DIR = Path(__file__).resolve().parent / "weights"


def layer_shapes() -> list[tuple[int, int]]:
    L = abi.lib()
    out = []
    ci, co = C.c_uint32(), C.c_uint32()
    layer = 0
    while L.pt_unet_layer_shape(layer, C.byref(ci), C.byref(co)):
        out.append((ci.value, co.value))
        layer += 1
    return out


def param_count() -> int:
    return int(abi.lib().pt_unet_param_count())


def init_params(seed: int = 0) -> np.ndarray:
    """He-normal weights (fan-in 9 * c_in), zero biases; the output layer is
    scaled by 0.02 (the network starts close to the identity on its
    residual base) and its channels 3..15 (unused) are zero."""
    rng = np.random.default_rng(seed)
    shapes = layer_shapes()
    parts = []
    for li, (ci, co) in enumerate(shapes):
        w = rng.standard_normal((9, ci, co)) * np.sqrt(2.0 / (9 * ci))
        if li == len(shapes) - 1:
            w *= 0.02
            w[:, :, 3:] = 0.0
        parts += [w.ravel(), np.zeros(co)]
    return np.concatenate(parts).astype(np.float32)


def save_params(path: Path, params: np.ndarray) -> None:
    """Parameters as raw little-endian float32 (the library's order)."""
    np.ascontiguousarray(params, dtype="<f4").tofile(path)


def load_params(path: Path) -> np.ndarray:
    p = np.fromfile(path, dtype="<f4")
    if p.size != param_count():
        raise ValueError(f"{path}: {p.size} parameters, the network has {param_count()}")
    return p


_TYPESTR = {"bfloat16": "<i2", "int16": "<i2", "float32": "<f4", "float64": "<f8", "uint8": "|u1"}


def device_tensor(ptr: int, shape, dtype):
    """A torch tensor viewing `ptr` (device memory owned by the library).
    bfloat16 views are made through int16 storage."""
    import torch

    name = str(dtype).replace("torch.", "")

    class _View:
        __cuda_array_interface__ = {"data": (int(ptr), False), "shape": tuple(shape), "typestr": _TYPESTR[name],
                                    "version": 2}

    t = torch.as_tensor(_View(), device="cuda")
    return t.view(torch.bfloat16) if name == "bfloat16" else t


class UNet:
    """A native U-Net for batch x height x width (sides multiples of 8)."""

    def __init__(self, batch: int, height: int, width: int, device: int = 0):
        L = abi.lib()
        self._lib = L
        self._h = L.pt_unet_create(device, batch, height, width)
        if not self._h:
            raise abi.PtError(abi.PT_ERR_INVALID, L.pt_unet_last_error(None).decode())
        self.batch, self.height, self.width = batch, height, width

    def _check(self, rc: int) -> None:
        if rc != abi.PT_OK:
            raise abi.PtError(rc, self._lib.pt_unet_last_error(self._h).decode())

    def close(self) -> None:
        if self._h:
            self._lib.pt_unet_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    @property
    def input_ptr(self) -> int:
        return int(self._lib.pt_unet_input(self._h))

    @property
    def output_ptr(self) -> int:
        return int(self._lib.pt_unet_output(self._h))

    def input_tensor(self):
        """The network's input buffer as a torch bfloat16 [batch, h, w, 16] view."""
        import torch

        return device_tensor(self.input_ptr, (self.batch, self.height, self.width, 16), torch.bfloat16)

    def output_tensor(self):
        """The last forward pass's fp32 [batch, h, w, 16] output (a view)."""
        import torch

        return device_tensor(self.output_ptr, (self.batch, self.height, self.width, 16), torch.float32)

    def base_tensor(self):
        """The fp32 [batch, h, w, 4] residual base added to output channels 0-3."""
        import torch

        return device_tensor(int(self._lib.pt_unet_base(self._h)), (self.batch, self.height, self.width, 4), torch.float32)

    def set_params(self, params: np.ndarray) -> None:
        p = np.ascontiguousarray(params, dtype=np.float32)
        self._check(self._lib.pt_unet_set_params(self._h, p.ctypes.data_as(C.POINTER(C.c_float)), p.size))

    def params(self) -> np.ndarray:
        p = np.empty(param_count(), np.float32)
        self._check(self._lib.pt_unet_get_params(self._h, p.ctypes.data_as(C.POINTER(C.c_float)), p.size))
        return p

    def grads(self) -> np.ndarray:
        g = np.empty(param_count(), np.float32)
        self._check(self._lib.pt_unet_get_grads(self._h, g.ctypes.data_as(C.POINTER(C.c_float)), g.size))
        return g

    def adam_state(self) -> tuple[np.ndarray, np.ndarray, int]:
        """(first moments, second moments, Adam steps taken)."""
        m, v = np.empty(param_count(), np.float32), np.empty(param_count(), np.float32)
        t = C.c_uint32(0)
        self._check(self._lib.pt_unet_get_adam_state(self._h, m.ctypes.data_as(C.POINTER(C.c_float)),
                                                      v.ctypes.data_as(C.POINTER(C.c_float)), m.size, C.byref(t)))
        return m, v, int(t.value)

    def set_adam_state(self, m: np.ndarray, v: np.ndarray, step: int) -> None:
        """Puts optimizer state back (after set_params, which clears it)."""
        m = np.ascontiguousarray(m, np.float32)
        v = np.ascontiguousarray(v, np.float32)
        self._check(self._lib.pt_unet_set_adam_state(self._h, m.ctypes.data_as(C.POINTER(C.c_float)),
                                                      v.ctypes.data_as(C.POINTER(C.c_float)), m.size, step))

    def forward(self, output_ptr: int | None = None, stream: int | None = None) -> None:
        self._check(self._lib.pt_unet_forward(self._h, output_ptr, stream))

    def backward(self, target_ptr: int, stream: int | None = None) -> float:
        loss = C.c_double()
        self._check(self._lib.pt_unet_backward(self._h, target_ptr, C.byref(loss), stream))
        return loss.value

    def adam(self, lr: float, stream: int | None = None) -> None:
        self._check(self._lib.pt_unet_adam(self._h, lr, stream))
