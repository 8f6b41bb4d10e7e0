"""The observables oracle against the reference's own analysis
(tests/golden/order_2d.npz, made by tests/golden/make_order_golden.py from
analysis/afa/utils.py compute_tangents and analysis/analyze_correlations.py
compute_relative_orientations).  No GPU."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import GOLDEN

import observables_oracle as obs


@pytest.fixture(scope="module")
def golden():
    return dict(np.load(GOLDEN / "order_2d.npz"))


def frames(g):
    return [str(x) for x in g["names"]]


def test_tangents_are_the_references(golden):
    for name in frames(golden):
        t = obs.tangents(golden[f"{name}_r"], int(golden[f"{name}_L"]))
        assert np.array_equal(t, golden[f"{name}_t"]), name


def test_relative_orientations_are_the_references(golden):
    for name in frames(golden):
        r, t = golden[f"{name}_r"], golden[f"{name}_t"]
        dist, nn, tt, S, P = obs.relative_orientations(r, t, golden[f"{name}_i"], golden[f"{name}_j"],
                                                       golden[f"{name}_box"])
        assert np.allclose(dist, golden[f"{name}_dist"], rtol=1e-6, atol=0), name
        assert np.array_equal(tt, golden[f"{name}_tt"]) and np.array_equal(nn, golden[f"{name}_nn"]), name
        assert abs(S - golden[f"{name}_S"]) < 1e-6 and abs(P - golden[f"{name}_P"]) < 1e-6, name


def test_order_parameters_over_all_beads_are_the_sampled_limit(golden):
    """order_parameters averages over every bead what the reference averages
    over its samples: with every index as the sample, the two agree; a planar
    frame's S also equals 1/4 + 3/4 S2D."""
    for name in frames(golden):
        r, t = golden[f"{name}_r"], golden[f"{name}_t"]
        every = np.arange(len(r))
        _, _, _, S, P = obs.relative_orientations(r, t, every, every, golden[f"{name}_box"])
        o = obs.order_parameters(t)
        # the reference-style average runs in float32 (7 digits), the oracle's in float64
        assert abs(o["s_q3"] - S) < 1e-5 and abs(o["polar"] - P) < 1e-5, name
        n, nt = len(t), o["n_tangents"]
        # Q over all beads counts the two beads without a tangent as t = 0
        planar = 0.25 + 0.75 * o["s_2d"] * nt / n
        assert abs(o["s_q3"] - planar) < 2e-3, (name, o["s_q3"], planar)


def test_bin_weights_partition_unity_and_are_smooth():
    d = np.linspace(0.2, 7.7, 20001)
    c, w = obs.bin_weights(d, 8.0, 32)
    assert np.allclose(w.sum(1), 1.0)
    # a fixed bin's weight is continuous across the centre changes: its
    # slope is at most 4 per unit distance (bins of 0.25), so no step of
    # 3.75e-4 changes it by more than 1.5e-3 (a jump would be ~0.1 or more)
    wb = np.zeros_like(d)
    for q in range(3):
        wb += np.where(c - 1 + q == 10, w[:, q], 0.0)
    assert np.abs(np.diff(wb)).max() < 2e-3
