"""Pipeline contract (reference: d2ic/dic_base.py:9-47): ``prepare(ref, assets)`` once, ``run(def)`` per frame."""
from __future__ import annotations

from abc import ABC, abstractmethod

from .dataclasses import DICResult
from .mesh_assets import MeshAssets
from .types import Array


class DICBase(ABC):
    @abstractmethod
    def prepare(self, ref_image: Array, assets: MeshAssets) -> None:
        raise NotImplementedError

    @abstractmethod
    def run(self, def_image: Array) -> DICResult:
        raise NotImplementedError
