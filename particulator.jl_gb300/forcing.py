"""Fields, forcings and pushers (pusher.jl, field.jl, continuum.jl).

The device integrates RK2Pusher(CombinedForcing(ElectromagneticField(E, B),
ChebContinuumLoss)) with a homogeneous B and an E that is homogeneous or one
of the position-dependent fields of field.jl (double layer, step, confined
double layer); these classes describe that pusher so that it can be handed to
``advance``/``run`` the way the reference takes its `pusher` argument.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from .tables import ChebContinuumLoss


@dataclass
class HomogeneousField:
    """HomogeneousField(v) (field.jl:4-8)."""
    v: tuple

    def __post_init__(self):
        self.v = tuple(float(a) for a in self.v)


@dataclass
class DoubleLayerField:
    """DoubleLayerField(z1, z2, v) (field.jl:10-16): v for z1 < z < z2, else 0."""
    z1: float
    z2: float
    v: tuple

    def device(self):
        return 1, [float(self.z1), float(self.z2)] + [float(a) for a in self.v]


@dataclass
class StepField:
    """StepField(z, v1, v2) (field.jl:19-27): v1 below z, v2 above."""
    z: float
    v1: tuple
    v2: tuple

    def device(self):
        return 2, [float(self.z)] + [float(a) for a in self.v1] + [float(a) for a in self.v2]


@dataclass
class ConfinedDoubleLayerField:
    """ConfinedDoubleLayerField(sx, sy, sz, ez0) (field.jl:30-52)."""
    sx: float
    sy: float
    sz: float
    ez0: float

    def device(self):
        return 3, [float(self.sx), float(self.sy), float(self.sz), float(self.ez0)]


@dataclass
class ElectromagneticField:
    """ElectromagneticField(e, b) (field.jl:54-70): force q (E + v x B)."""
    e: HomogeneousField
    b: HomogeneousField


class NullForcing:
    """NullForcing (pusher.jl:11)."""


class CombinedForcing:
    """CombinedForcing(a, b...) (pusher.jl:14-23)."""

    def __init__(self, *tpl):
        self.tpl = tpl


class RK2Pusher:
    """RK2Pusher(forcing) (pusher.jl:37-63), Ralston's 2/3 two-stage scheme."""

    def __init__(self, forcing):
        self.forcing = forcing

    def device_forcing(self):
        """(E, B, ChebContinuumLoss | None) the device integrates."""
        items = self.forcing.tpl if isinstance(self.forcing, CombinedForcing) else (self.forcing,)
        E = np.zeros(3)
        B = np.zeros(3)
        cl = None
        for f in items:
            if isinstance(f, ElectromagneticField):
                if not isinstance(f.b, HomogeneousField):
                    raise NotImplementedError("only a homogeneous B runs on the device")
                if isinstance(f.e, HomogeneousField):
                    E += np.array(f.e.v)
                elif not hasattr(f.e, "device"):
                    raise NotImplementedError(f"field {type(f.e).__name__} has no device implementation")
                B += np.array(f.b.v)
            elif isinstance(f, ChebContinuumLoss):
                if cl is not None:
                    raise NotImplementedError("one continuum-loss term at most")
                cl = f
            elif isinstance(f, NullForcing):
                pass
            else:
                raise NotImplementedError(f"forcing {type(f).__name__} has no device implementation")
        return E, B, cl

    def device_efield(self):
        """(kind, params) of the position-dependent E (pcl_set_field); kind 0
        when E is homogeneous."""
        items = self.forcing.tpl if isinstance(self.forcing, CombinedForcing) else (self.forcing,)
        found = [f.e for f in items if isinstance(f, ElectromagneticField) and hasattr(f.e, "device")]
        if not found:
            return 0, []
        if len(found) > 1 or np.any(self.device_forcing()[0] != 0):
            raise NotImplementedError("one position-dependent E and no homogeneous E beside it")
        return found[0].device()
