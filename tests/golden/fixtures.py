"""Loaders of the golden fixtures: scenes, views and pyramids in the reference layouts."""
from __future__ import annotations

from pathlib import Path

import numpy as np

from blitzen_gb300 import abi
from blitzen_gb300 import scenes as S

HERE = Path(__file__).resolve().parent


def load(name: str):
    return np.load(HERE / f"{name}.npz")


def scene(d) -> S.Scene:
    return S.Scene(d["objects"], d["transforms"], d["surfaces"], d["lods"],
                   visibility=d["visibility"] if "visibility" in d.files else None)


def view(raw: np.ndarray) -> abi.CameraViewData:
    v = abi.CameraViewData()
    b = np.ascontiguousarray(raw, np.uint8).tobytes()
    assert len(b) == 256
    abi.C.memmove(abi.C.addressof(v), b, 256)
    return v


def pyramid_desc(depth_w: int, depth_h: int, mode: int = abi.HIZ_D3D12) -> tuple[abi.Pyramid, int]:
    return abi.pyramid_layout(depth_w, depth_h, mode)
