"""Philox4x32-10 known answers: cuRAND's host Philox generator (a library run,
output comparison only) emits, for seed s, block j = Philox4x32-10 of counter
(0, 0, j, 0) under key (s lo, s hi)."""
from __future__ import annotations

import numpy as np
import pytest

import oracle_lib as O


@pytest.mark.parametrize("seed", [1234, 0x0123456789ABCDEF, 0])
def test_oracle_philox_matches_curand_host(seed):
    n_blocks = 512
    ref = O.curand_philox_u32(4 * n_blocks, seed).reshape(n_blocks, 4)
    mine = np.stack([O.philox((0, 0, j, 0), (seed & 0xFFFFFFFF, seed >> 32)) for j in range(n_blocks)])
    assert np.array_equal(mine, ref)


def test_host_normals_are_standard_normal():
    z = O.host_normals(1234, 0, 2000, 50, ).reshape(-1)
    assert abs(z.mean()) < 0.01
    assert abs(z.std() - 1.0) < 0.01
    # Box-Muller of 24-bit uniforms: bounded by sqrt(-2 log 2^-24) ~ 5.77
    assert np.max(np.abs(z)) < 5.8
