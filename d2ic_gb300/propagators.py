"""Warm-start propagators (reference: d2ic/propagator_base.py, propagator_previous.py,
propagator_constant_velocity.py).  Work on numpy arrays and torch tensors alike."""
from __future__ import annotations

from abc import ABC, abstractmethod
from typing import Optional

from .types import Array


class DisplacementPropagatorBase(ABC):
    @abstractmethod
    def propagate(self, u_prev: Optional[Array], u_prevprev: Optional[Array] = None) -> Optional[Array]:
        raise NotImplementedError


class PreviousDisplacementPropagator(DisplacementPropagatorBase):
    """``u_warm = u_prev``."""

    def propagate(self, u_prev, u_prevprev=None):
        return u_prev


class ConstantVelocityPropagator(DisplacementPropagatorBase):
    """``u_warm = 2 u_prev - u_prevprev``; ``u_prev`` alone if there is no second history frame."""

    def propagate(self, u_prev, u_prevprev=None):
        if u_prev is None:
            return None
        if u_prevprev is None:
            return u_prev
        return 2.0 * u_prev - u_prevprev
