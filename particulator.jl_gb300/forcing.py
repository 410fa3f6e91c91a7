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


_SPECIES = {"electron": 0, "photon": 1, "positron": 2}


def _species_bit(particle) -> int:
    return 1 << (_SPECIES[particle.lower()] if isinstance(particle, str) else int(particle))


class RestrictedForcing:
    """RestrictedForcing{T}(f) (pusher.jl:28-34): f acts on species T only
    (the field or the continuum loss of one species, e.g. losses for
    positrons alone)."""

    def __init__(self, particle, forcing):
        self.bit = _species_bit(particle)
        self.forcing = forcing


def _leaves(forcing, mask=7):
    """(forcing, species mask) of every leaf of a combined / restricted
    forcing."""
    if isinstance(forcing, CombinedForcing):
        for f in forcing.tpl:
            yield from _leaves(f, mask)
    elif isinstance(forcing, RestrictedForcing):
        yield from _leaves(forcing.forcing, mask & forcing.bit)
    else:
        yield forcing, mask


class RK2Pusher:
    """RK2Pusher(forcing) (pusher.jl:37-63), Ralston's 2/3 two-stage scheme."""

    def __init__(self, forcing):
        self.forcing = forcing

    def device_masks(self):
        """(pushed, field, loss): the species bits pushed at all, feeling the
        EM field, feeling the continuum loss (pcl_set_push_mask).  Every EM
        field acts on the same species, and there is one loss term at most."""
        field, loss = None, 7
        for f, m in _leaves(self.forcing):
            if isinstance(f, ElectromagneticField):
                if field is not None and field != m:
                    raise NotImplementedError("EM fields restricted to different species")
                field = m
            elif isinstance(f, ChebContinuumLoss):
                loss = m
        return 7, (7 if field is None else field), loss

    def device_forcing(self):
        """(E, B, ChebContinuumLoss | None) the device integrates."""
        items = [f for f, _ in _leaves(self.forcing)]
        E = np.zeros(3)
        B = np.zeros(3)
        cl = None
        for f in items:
            if isinstance(f, ElectromagneticField):
                for g in (f.e, f.b):
                    if not isinstance(g, HomogeneousField) and not hasattr(g, "device"):
                        raise NotImplementedError(f"field {type(g).__name__} has no device implementation")
                if isinstance(f.e, HomogeneousField):
                    E += np.array(f.e.v)
                if isinstance(f.b, HomogeneousField):
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
        items = [f for f, _ in _leaves(self.forcing)]
        found = [f.e for f in items if isinstance(f, ElectromagneticField) and hasattr(f.e, "device")]
        if not found:
            return 0, []
        if len(found) > 1 or np.any(self.device_forcing()[0] != 0):
            raise NotImplementedError("one position-dependent E and no homogeneous E beside it")
        return found[0].device()

    def device_bfield(self):
        """(kind, params) of the position-dependent B (pcl_set_bfield), in T;
        kind 0 when B is homogeneous."""
        items = [f for f, _ in _leaves(self.forcing)]
        found = [f.b for f in items if isinstance(f, ElectromagneticField) and hasattr(f.b, "device")]
        if not found:
            return 0, []
        if len(found) > 1 or np.any(self.device_forcing()[1] != 0):
            raise NotImplementedError("one position-dependent B and no homogeneous B beside it")
        return found[0].device()


class RestrictedPusher:
    """RestrictedPusher{T}(p) (pusher.jl:67-73): p advances species T; the
    other species only advance their clocks (no motion, photons included)."""

    def __init__(self, particle, pusher):
        self.bit = _species_bit(particle)
        self.pusher = pusher

    def device_masks(self):
        push, field, loss = self.pusher.device_masks()
        return push & self.bit, field, loss

    def device_forcing(self):
        return self.pusher.device_forcing()

    def device_efield(self):
        return self.pusher.device_efield()

    def device_bfield(self):
        return self.pusher.device_bfield()


class NullPusher:
    """NullPusher (pusher.jl:75-76): no particle moves; clocks advance, and
    collisions happen as the null-collision clock says."""

    def device_masks(self):
        return 0, 7, 7

    def device_forcing(self):
        return np.zeros(3), np.zeros(3), None

    def device_efield(self):
        return 0, []

    def device_bfield(self):
        return 0, []
