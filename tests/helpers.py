"""Shared helpers of the parity tests: scene upload, GPU runs through the C ABI, oracle runs."""
from __future__ import annotations

import numpy as np

from blitzen_gb300 import abi
from blitzen_gb300 import scenes as S

W, H = 1920, 1080


def view_for(zfar=1e4, position=(0.0, 0.0, 0.0), yaw=0.0, pitch=0.0, pw=960.0, ph=540.0, width=W, height=H):
    return abi.view_setup(S.fov_radians(), float(width), float(height), S.ZNEAR, zfar, position, yaw, pitch, pw, ph)


def assert_records_equal(gpu: tuple[int, np.ndarray], ref: tuple[int, np.ndarray], what: str = ""):
    """Draw counts and every word of every stored record, the 32-byte form's two pad words included
    (neither side writes them: both buffers start zeroed)."""
    gn, gr = gpu
    rn, rr = ref
    assert gn == rn, f"{what}: draw count {gn} != oracle {rn}"
    assert gr.shape == rr.shape, f"{what}: stored {gr.shape} != {rr.shape}"
    if gr.size:
        bad = np.nonzero((gr != rr).any(axis=1))[0]
        assert bad.size == 0, f"{what}: {bad.size} records differ, first at {bad[0]}: {gr[bad[0]]} vs {rr[bad[0]]}"
