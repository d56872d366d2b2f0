"""Solver plugin contract (reference: d2ic/solver_base.py:8-26)."""
from __future__ import annotations

from abc import ABC, abstractmethod
from typing import Any

from .types import Array


class SolverBase(ABC):
    """A solver owns its preparation (``compile``) and its per-frame loop (``solve``)."""

    @abstractmethod
    def compile(self, assets: Any) -> None:
        raise NotImplementedError

    @abstractmethod
    def solve(self, state: Any, def_image: Array) -> Any:
        raise NotImplementedError
