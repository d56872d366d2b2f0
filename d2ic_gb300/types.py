"""Type aliases (reference: d2ic/types.py)."""
from __future__ import annotations

from typing import Any, Tuple

import numpy as np

Array = Any          # numpy array or torch tensor
NPArray = np.ndarray
XY = Tuple[float, float]
