"""Fields, forcings and pushers (pusher.jl, field.jl, continuum.jl).

The device integrates RK2Pusher(CombinedForcing(ElectromagneticField(E, B),
ChebContinuumLoss)) with homogeneous E and B; these classes describe that
pusher so that it can be handed to ``advance``/``run`` the way the reference
takes its `pusher` argument.
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
                if not isinstance(f.e, HomogeneousField) or not isinstance(f.b, HomogeneousField):
                    raise NotImplementedError("only homogeneous fields run on the device")
                E += np.array(f.e.v)
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
