"""Host-side handle of the learned depth refiner (include/tde_refiner.h).

Device buffers are passed as integer addresses (e.g. ``tensor.data_ptr()``);
the convenience methods taking numpy arrays copy through torch CUDA tensors.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._capi import check, declare, lib

P, I, F, SZ = C.c_void_p, C.c_int, C.c_float, C.c_size_t

declare("tde_refiner_create", I, [I, I, I, C.c_uint64, C.POINTER(P)])
declare("tde_refiner_destroy", I, [P])
declare("tde_refiner_param_count", SZ, [])
declare("tde_refiner_get_params", I, [P, P, SZ])
declare("tde_refiner_set_params", I, [P, P, SZ])
declare("tde_refiner_set_adamw", I, [P, F, F, F, F])
declare("tde_refiner_forward", I, [P, P, I, P, P, P])
declare("tde_refiner_loss_grad", I, [P, P, P, I, P])
declare("tde_refiner_train_step", I, [P, P, P, I, F, P])
declare("tde_refiner_get_grads", I, [P, P, SZ])
declare("tde_refiner_last_loss", I, [P, C.POINTER(C.c_double), C.POINTER(C.c_double)])
declare("tde_refiner_get_tensor", I, [P, I, P, SZ])
declare("tde_refiner_tensor_bytes", SZ, [P, I])
declare("tde_refiner_status", I, [P])
declare("tde_wait_selftest", I, [C.c_uint64, P, P])

ACTIVATIONS = ["e0a", "e0", "e1a", "e1", "e2a", "e2", "b3a", "b3", "d2", "d1", "d0"]
GRADIENTS = ["dz11", "gu0", "dz10", "gu1", "dz9", "gu2", "dz8", "dz7", "gp3", "dz6", "dz5", "gp2", "dz4", "dz3",
             "gp1", "dz2", "dz1"]
TENSOR_IDS = {n: i for i, n in enumerate(ACTIVATIONS)}
TENSOR_IDS["out"] = len(ACTIVATIONS)
TENSOR_IDS.update({n: len(ACTIVATIONS) + 1 + i for i, n in enumerate(GRADIENTS)})
CHANNELS = {"e0a": 16, "e0": 16, "e1a": 32, "e1": 32, "e2a": 48, "e2": 48, "b3a": 64, "b3": 64, "d2": 48,
            "d1": 32, "d0": 16, "dz11": 16, "gu0": 48, "dz10": 32, "gu1": 80, "dz9": 48, "gu2": 112, "dz8": 64,
            "dz7": 64, "gp3": 48, "dz6": 48, "dz5": 48, "gp2": 32, "dz4": 32, "dz3": 32, "gp1": 16, "dz2": 16,
            "dz1": 16}

LEVELS = {"e0a": 0, "e0": 0, "e1a": 1, "e1": 1, "e2a": 2, "e2": 2, "b3a": 3, "b3": 3, "d2": 2, "d1": 1, "d0": 0,
          "dz11": 0, "gu0": 0, "dz10": 1, "gu1": 1, "dz9": 2, "gu2": 2, "dz8": 3, "dz7": 3, "gp3": 3, "dz6": 2,
          "dz5": 2, "gp2": 2, "dz4": 1, "dz3": 1, "gp1": 1, "dz2": 0, "dz1": 0}


# The tensor-core convolutions c2..c11: (pyramid level, input channels, output channels).
CONVS = [(0, 16, 16), (1, 16, 32), (1, 32, 32), (2, 32, 48), (2, 48, 48), (3, 48, 64), (3, 64, 64), (2, 112, 48),
         (1, 80, 32), (0, 48, 16)]


def conv_flops(rows: int, cols: int, batch: int = 1, train: bool = False) -> int:
    """Multiply-add FLOPs (2 per MAC) of the tensor-core convolutions of one
    forward pass, or of a training step (forward, input gradients and weight
    gradients: three times as many)."""
    f = sum(2 * (rows >> l) * (cols >> l) * 9 * ci * co for l, ci, co in CONVS) * batch
    return 3 * f if train else f


def param_count() -> int:
    return int(lib.tde_refiner_param_count())


class Refiner:
    def __init__(self, max_batch: int, rows: int, cols: int, seed: int = 0):
        h = P()
        check(lib.tde_refiner_create(max_batch, rows, cols, seed, C.byref(h)))
        self._h = h
        self.max_batch, self.rows, self.cols = max_batch, rows, cols

    @property
    def handle(self):
        return self._h

    def close(self):
        if self._h:
            lib.tde_refiner_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- parameters --------------------------------------------------------
    def get_params(self) -> np.ndarray:
        a = np.zeros(param_count(), np.float32)
        check(lib.tde_refiner_get_params(self._h, a.ctypes.data_as(P), a.size))
        return a

    def set_params(self, theta: np.ndarray) -> None:
        a = np.ascontiguousarray(theta, np.float32)
        check(lib.tde_refiner_set_params(self._h, a.ctypes.data_as(P), a.size))

    def set_adamw(self, beta1=0.9, beta2=0.999, eps=1e-8, weight_decay=0.01) -> None:
        check(lib.tde_refiner_set_adamw(self._h, beta1, beta2, eps, weight_decay))

    # -- device-pointer API -----------------------------------------------
    def forward_ptr(self, raw, batch, out_mm=0, out_m=0, stream=0) -> None:
        check(lib.tde_refiner_forward(self._h, raw, batch, out_mm or None, out_m or None, stream or None))

    def loss_grad_ptr(self, raw, target, batch, stream=0) -> None:
        check(lib.tde_refiner_loss_grad(self._h, raw, target, batch, stream or None))

    def train_step_ptr(self, raw, target, batch, lr, stream=0) -> None:
        check(lib.tde_refiner_train_step(self._h, raw, target, batch, lr, stream or None))

    # -- results --------------------------------------------------------------
    def grads(self) -> np.ndarray:
        a = np.zeros(param_count(), np.float32)
        check(lib.tde_refiner_get_grads(self._h, a.ctypes.data_as(P), a.size))
        return a

    def last_loss(self):
        loss, cnt = C.c_double(), C.c_double()
        check(lib.tde_refiner_last_loss(self._h, C.byref(loss), C.byref(cnt)))
        return loss.value, cnt.value

    def tensor(self, name: str) -> np.ndarray:
        """An internal tensor of the last call, as float32 [batch, h, w(, c)]."""
        tid = TENSOR_IDS[name]
        nbytes = int(lib.tde_refiner_tensor_bytes(self._h, tid))
        if nbytes == 0:
            raise ValueError("no tensor yet")
        if name == "out":
            a = np.zeros(nbytes // 4, np.float32)
            check(lib.tde_refiner_get_tensor(self._h, tid, a.ctypes.data_as(P), nbytes))
            return a.reshape(-1, self.rows, self.cols)
        u = np.zeros(nbytes // 2, np.uint16)
        check(lib.tde_refiner_get_tensor(self._h, tid, u.ctypes.data_as(P), nbytes))
        f = (u.astype(np.uint32) << 16).view(np.float32)
        lv, c = LEVELS[name], CHANNELS[name]
        return f.reshape(-1, self.rows >> lv, self.cols >> lv, c)

    def status(self) -> int:
        """0, or TDE_ERR_DEVICE_TIMEOUT once a tensor-core wait gave up (synchronises)."""
        return lib.tde_refiner_status(self._h)

    def check_status(self) -> None:
        """Raises TdeError when a tensor-core wait of an earlier launch gave up."""
        check(self.status())

    # -- numpy conveniences (copies through torch) ---------------------------
    def forward(self, raw_mm: np.ndarray):
        import torch
        raw = torch.from_numpy(np.ascontiguousarray(raw_mm, np.uint16).view(np.int16)).cuda()
        n = raw.shape[0]
        out_mm = torch.zeros_like(raw)
        out_m = torch.zeros(raw.shape, dtype=torch.float32, device=raw.device)
        self.forward_ptr(raw.data_ptr(), n, out_mm.data_ptr(), out_m.data_ptr())
        torch.cuda.synchronize()
        return out_mm.cpu().numpy().view(np.uint16), out_m.cpu().numpy()

    def loss_grad(self, raw_mm: np.ndarray, target_mm: np.ndarray):
        import torch
        raw = torch.from_numpy(np.ascontiguousarray(raw_mm, np.uint16).view(np.int16)).cuda()
        tgt = torch.from_numpy(np.ascontiguousarray(target_mm, np.uint16).view(np.int16)).cuda()
        self.loss_grad_ptr(raw.data_ptr(), tgt.data_ptr(), raw.shape[0])
        torch.cuda.synchronize()
        return self.last_loss()[0], self.grads()
