"""The part cost model (the reference's src/part.ts:7-29)."""
from __future__ import annotations

import math

K_RV = 0.3


def rv_cost(mesh_vol: float, hull_vol: float) -> float:
    """0.3 * cbrt(3/(4 pi) * max(hullVol - meshVol, 0))  (part.ts:24-26)."""
    return K_RV * math.cbrt((3 / (4 * math.pi)) * max(hull_vol - mesh_vol, 0.0))


def part_cost(mesh_vol: float, hull_vol: float, hausdorff) -> float:
    """max(rv, hausdorff) (part.ts:27-29); a missing Hausdorff counts as 0."""
    return max(rv_cost(mesh_vol, hull_vol), hausdorff or 0.0)
