"""The learned inverse-CDF sampler: a small network trained on samples of the
table samplers (Seltzer-Berger photon energy, Moller secondary energy) and used
by the step in place of them inside its trained range.

Inputs a = (log10(T / eV) - 6) / 2 for T in [1e4, 1e8] eV, b = 2u - 1.
Outputs: bremsstrahlung y = ln(k / T); Moller v with
eps = e0 / (1 - v (1 - 2 e0)), e0 = tcut / T (v is the proposal's uniform of
moller.jl:70, so v ~ u where the rejection accepts everything).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from . import constants as co

T_MIN_EV, T_MAX_EV = 1e4, 1e8
LEARN_SB, LEARN_MOLLER = 1, 2


def features(T, u) -> np.ndarray:
    """(n, 2) float32 network inputs for kinetic energies T (J) and uniforms u."""
    a = (np.log10(np.asarray(T, dtype=float) / co.eV) - 6.0) / 2.0
    b = 2.0 * np.asarray(u, dtype=float) - 1.0
    return np.ascontiguousarray(np.stack(np.broadcast_arrays(a, b), axis=-1), dtype=np.float32)


class SamplerNet:
    """Device handle of one network (pcl_mlp_*)."""

    def __init__(self, device: int = 0, seed: int = 0):
        h = C.c_void_p()
        rc = _lib.lib().pcl_mlp_create(int(device), int(seed), C.byref(h))
        if rc != _lib.PCL_OK:
            raise _lib.PCLError(rc, "pcl_mlp_create failed (is a CUDA device available?)")
        self.h = h

    def _check(self, rc, what):
        if rc != _lib.PCL_OK:
            raise _lib.PCLError(rc, f"{what}: {_lib.lib().pcl_mlp_last_error(self.h).decode(errors='replace')}")

    def params(self) -> np.ndarray:
        p = np.zeros(_lib.MLP_NPARAM, np.float32)
        self._check(_lib.lib().pcl_mlp_get_params(self.h, _lib.fptr(p), len(p)), "pcl_mlp_get_params")
        return p

    def set_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        self._check(_lib.lib().pcl_mlp_set_params(self.h, _lib.fptr(p), len(p)), "pcl_mlp_set_params")

    def forward(self, x) -> np.ndarray:
        x = np.ascontiguousarray(x, dtype=np.float32).reshape(-1, 2)
        y = np.zeros(len(x), np.float32)
        self._check(_lib.lib().pcl_mlp_forward(self.h, len(x), _lib.fptr(x), _lib.fptr(y)), "pcl_mlp_forward")
        return y

    def gradient(self, x, t):
        x = np.ascontiguousarray(x, dtype=np.float32).reshape(-1, 2)
        t = np.ascontiguousarray(t, dtype=np.float32)
        g = np.zeros(_lib.MLP_NPARAM, np.float32)
        loss = C.c_double()
        self._check(_lib.lib().pcl_mlp_gradient(self.h, len(x), _lib.fptr(x), _lib.fptr(t), _lib.fptr(g),
                                                C.byref(loss)), "pcl_mlp_gradient")
        return g, loss.value

    def train(self, x, t, steps: int, batch: int = 8192, lr: float = 2e-3, seed: int = 0) -> float:
        x = np.ascontiguousarray(x, dtype=np.float32).reshape(-1, 2)
        t = np.ascontiguousarray(t, dtype=np.float32)
        loss = C.c_double()
        self._check(_lib.lib().pcl_mlp_train(self.h, len(x), _lib.fptr(x), _lib.fptr(t), int(steps), int(batch),
                                             float(lr), int(seed), C.byref(loss)), "pcl_mlp_train")
        return loss.value

    def close(self):
        if getattr(self, "h", None):
            _lib.lib().pcl_mlp_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
