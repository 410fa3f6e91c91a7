"""The learned inverse-CDF sampler: a small network trained on samples of the
table samplers (Seltzer-Berger photon energy, Moller secondary energy) and used
by the step in place of them inside its trained range.

Inputs a = (log10(T / eV) - 6) / 2 for T in [1e4, 1e8] eV, b = 2u - 1.
Outputs, both in [0, 1] and increasing in u: bremsstrahlung h with
ln(k / T) = (1 - h) ln(kmin / T), kmin / T the Seltzer-Berger table's pcum = 0
value at T; Moller v with eps = e0 / (1 - v (1 - 2 e0)), e0 = tcut / T (v is
the proposal's uniform of moller.jl:70, so v ~ u where the rejection accepts
everything).
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


def learn_data(mpopl, species: int, proc_index: int, kind: int, *, samples: float = 1e8, nT: int = 1024,
               Q: int = 1024, seed: int = 0):
    """Training set of the network for table position `proc_index` of
    `species` in `mpopl` (pcl_learn_data): `samples` draws of the table sampler
    spread over nT energies, turned into Q quantile targets per energy.
    Returns (x (rows, 2) float32, t (rows,) float32)."""
    per_T = max(1, int(samples // nT))
    x = np.zeros((nT * Q, 2), np.float32)
    t = np.zeros(nT * Q, np.float32)
    rows = C.c_int64()
    _lib.check(_lib.lib().pcl_learn_data(mpopl.ctx, int(species), int(proc_index), int(kind), int(nT), per_T, int(Q),
                                         int(seed), _lib.fptr(x), _lib.fptr(t), C.byref(rows)),
               mpopl.ctx, "pcl_learn_data")
    return x[:rows.value], t[:rows.value]


def train_sampler(mpopl, species: int, proc_index: int, kind: int, *, samples: float = 1e8, nT: int = 1024,
                  Q: int = 1024, steps: int = 8000, batch: int = 8192, lr: float = 2e-3, seed: int = 0,
                  device: int = 0):
    """Generate the training set on the device from the table sampler and
    train a network on it with the tensor-core kernels.  Returns (net, loss)."""
    x, t = learn_data(mpopl, species, proc_index, kind, samples=samples, nT=nT, Q=Q, seed=seed)
    net = SamplerNet(device=device, seed=seed)
    loss = net.train(x, t, steps=steps, batch=batch, lr=lr, seed=seed)
    return net, loss


def table_positions(tab, kind: int):
    """Table positions of a collision table whose process the kind replaces."""
    from .processes import Moller, SeltzerBerger
    cls = SeltzerBerger if kind == LEARN_SB else Moller
    return [j for j, p in enumerate(tab.proc) if isinstance(p, cls)]


def sb_ymin(sb, T):
    """Lower bound of ln(k / T) of a SeltzerBerger table at kinetic energies
    T (J), as the device computes it: the pcum = 0 column, linear in ln T
    between grid energies, lowered by the column's largest step."""
    le = np.asarray(sb.log_energy)
    col = np.asarray(sb.data).reshape(len(le), -1)[:, 0]
    return np.interp(np.log(np.asarray(T, dtype=float)), le, col) - np.max(np.abs(np.diff(col)))
