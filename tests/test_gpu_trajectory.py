"""Trajectory frames: what the writer puts in the file is the state the
system reports at that step (6 significant digits, the reference's stream
formatting), with the reference's header keys, labels A for beads and B for
solvent, frames appended in order while the system keeps stepping."""
from __future__ import annotations

import numpy as np
import pytest

from nwgb import abi
from nwgb.init import initial_state, wca_config
from nwgb.trajectory import read_frames

pytestmark = pytest.mark.gpu

KEYS = ["iteration", "dt", "time", "num_particles", "num_filaments", "filament_size", "bond_spring_coef",
        "bond_spring_length", "bond_bending_coef", "activity", "kbT", "gamma", "particle_radius", "particle_mass",
        "num_cells", "grid_size", "box_size", "cell_size", "boundaries", "reverse_probability",
        "collision_spring_coef", "collision_damping_coef", "collision_shear_coef", "collision_attraction_coef",
        "boundary_damping_coef"]


def close6(a, b):
    # %g keeps 6 significant digits: half a unit of the 6th digit, relative
    return np.all(np.abs(a - b) <= 5e-6 * np.maximum(np.abs(b), 1e-30) + 1e-37)


def test_frames_match_the_state_at_each_step(lib, tmp_path):
    import nwgb

    cfg = wca_config(40, 10, (30.0, 30.0), srd=True, seed=4, lib=lib)
    pos, vel = initial_state(cfg, seed=4)
    path = tmp_path / "traj.xyzv"
    want = []
    with nwgb.System(cfg) as s:
        s.set_array(abi.NW_POSITION, pos)
        s.set_array(abi.NW_VELOCITY, vel)
        with s.writer(path) as w:
            for it in (0, 7, 20):
                if it > s.step_index:
                    s.step(it - s.step_index, cfg.dt)
                w.frame(it, cfg.dt)
                s.sync()
                want.append((it, s.get_array(abi.NW_POSITION), s.get_array(abi.NW_VELOCITY)))
                s.step(3, cfg.dt)  # the step loop runs on while the frame is written
            w.flush()
    frames = list(read_frames(path))
    assert len(frames) == 3
    nb, n = cfg.n_beads, cfg.n_beads + cfg.n_solvent
    for f, (it, p, v) in zip(frames, want):
        h = f["header"]
        assert list(h.keys()) == KEYS
        assert h["iteration"] == it and h["num_particles"] == nb and h["filament_size"] == cfg.filament_size
        assert abs(h["time"] - it * cfg.dt) < 1e-6
        assert f["pos"].shape == (n, 3)
        assert np.all(f["labels"][:nb] == "A") and np.all(f["labels"][nb:] == "B")
        assert close6(f["pos"], p[:, :3].astype(np.float64))
        assert close6(f["vel"], v[:, :3].astype(np.float64))


def test_writer_reports_an_unwritable_path(lib):
    import nwgb

    cfg = wca_config(4, 5, (10.0, 10.0), lib=lib)
    with nwgb.System(cfg) as s:
        with pytest.raises(nwgb.NwError) as e:
            s.writer("/nonexistent-dir/x.xyzv")
        assert e.value.status == abi.NW_ERR_IO
