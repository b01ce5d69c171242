"""Helpers to replay golden fixtures (made by tests/golden/make_golden.py)."""
from __future__ import annotations

import json
import os
from types import SimpleNamespace

import numpy as np

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")

SMALL = ["s8_upwind", "s16x12_quick", "s5x9_quick", "s12x10_nopc", "s9x7_noadv", "s6x6_nolid",
         "s3x4_tiny", "s2x2_min", "s16_patch"]


def load(name):
    return np.load(os.path.join(HERE, name + ".npz"))


def config_of(g):
    return SimpleNamespace(**json.loads(str(g["config"])))


def initial_interior(name, nx, ny):
    """Initial (u, v) of a fixture (zero except the patch case)."""
    u = np.zeros((ny, nx))
    v = np.zeros((ny, nx))
    if name == "s16_patch":
        u[4:10, 4:10] = 1.0
    return u, v


def fixture_platform(g):
    return json.loads(str(g["meta"]))
