#!/usr/bin/env python
"""bench.py — bead-steps/s of the nematic-worm step on GB300.

Workload (default): 2D WCA worms with SRD solvent, 20,000 worms x 20 beads =
400,000 beads in a periodic 1000 x 1000 box, 4,000,000 SRD particles (density
4 per unit cell), SRD collision every 10 steps, FP32, dt = 0.005.  A step is
one ParticleSystem::update equivalent (the SRD sub-step every 10th step).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Our arm: exactly W warm-up steps, then K steps replayed from CUDA graphs of 10
steps (one SRD period; every graph the timed region replays is captured
beforehand), timed with CUDA events on the engine's stream between a barrier +
synchronize on both sides; the timed region is repeated three times from the
same checkpoint and `value` is the median (`timing` gives all three).  The
state (~190 MB) is larger than L2.  Under torchrun every rank runs an
independent replica ("replicas only": a single system is not sharded) and
`value` is the sum over ranks.  Sub-blocks of the same line: `strategies`
(the same workload under the sorted-scheme, cell-list and Verlet strategies),
`reference_cuda` (the reference's own CUDA build against this engine's
REF_DEM model on the reference-feasible stand-in: 20,000 x 20 beads on a
1024 x 1024 grid with the reference's SRD, 2,621,440 solvent), `batch_256` and
`adjoint_64x4k`.  Reference arm (--impl reference): the CPU port of the
reference's step (oracle/, FP64, all host threads) on the same workload; it
does not load libnwgb.

Other workloads (--workload): wca_dense_2m (2M beads, no solvent),
wca_small_4k (4k beads), batch_256 (256 uneven replicas in one launch per
step), adjoint_64x4k (differentiable 200-step rollout of 64 replicas) and
defects_400k (the +1/2 / -1/2 defect searches on a 400k-bead frame).
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import time
from pathlib import Path

REPO = Path(__file__).resolve().parent
sys.path.insert(0, str(REPO / "nematic-worms_gb300"))

GAP = 10
GRAPH_STEPS = 100  # updates per step call (one CUDA graph each): whole SRD periods
assert GRAPH_STEPS % GAP == 0
REPEATS = 3
PEAKS_FILE = REPO / "MEASURED_PEAKS.json"
TRAFFIC_FILE = REPO / "profiles" / "traffic_per_unit.txt"
FALLBACK_HBM_GBS = 6800.0

WORKLOADS = {
    "wca_srd_400k": dict(k=1, layout="patches"),
    "wca_dense_2m": dict(k=2, layout="rows"),
    "wca_small_4k": dict(k=0, layout="patches"),
    # 256 replicas of uneven size (50-2000 worms x 5-30 beads, F_act 0-2,
    # k_bend 1-20, packing 0.3-0.6) in one batched launch per step
    "batch_256": dict(batch=256),
    # 64 replicas of the 4k-bead workload, 200-step differentiable rollout,
    # lists frozen per 20-step segment, gradient of the S / C_v loss
    "adjoint_64x4k": dict(adjoint=64),
    # +1/2 / -1/2 defect search on a 400,000-bead frame (40,000 worms x 10
    # beads, 8 planted defects, density 1 in a 632 x 632 box), cells of 2
    "defects_400k": dict(defects=(40000, 10, 632.0, 2.0)),
}


def env_rank():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("LOCAL_RANK", "0"))


# ---- algorithmic bytes per launch (reference float4 state model) -------------------
# Units of work and their compulsory bytes in the reference's float4 layout:
#   bead-step:  96 B (pos, vel, force read and written: 3 x 16 B each way)
#               + 16 B (one write and one read of the 8 B (key, value) pair)
#               + 8 C / N B (cell start/end written once and read once)
#   SRD collision, per solvent particle: 64 B (pos and vel read and written)
#               + 16 B (key, value) + 32 Cs / Ns B (cell momentum and energy sums)
BEAD_STEP_B = 112.0
SRD_PARTICLE_B = 80.0


def step_bytes(cfg) -> float:
    """Algorithmic bytes of one step: every bead-step plus the SRD collision
    amortised over its period."""
    b = cfg.n_beads * BEAD_STEP_B + 8.0 * cfg.n_cells
    if cfg.srd_enabled:
        b += (cfg.n_solvent * SRD_PARTICLE_B + 32.0 * cfg.n_srd_cells) / max(1, int(cfg.srd_gap))
    return b


def alg_bytes(name: str, cfg) -> float:
    """Compulsory DRAM bytes of one launch of kernel `name` in the units
    above: a kernel that completes a bead-step for every bead (the fused
    step kernel; the pair kernel of the sorted scheme, which finishes it)
    carries 112 N + 8 C; the collision kernel carries the collision's
    80 Ns + 32 Cs.  Kernels that only prepare a unit carry their own reads
    and writes (the sort's passes: 16 N over the pass, cell tables 8 C)."""
    nb, ns = cfg.n_beads, cfg.n_solvent
    C, Cs = cfg.n_cells, cfg.n_srd_cells
    step = 112.0 * nb + 8.0 * C
    table = {
        "bead_fused": step,
        "bead_epi": step,  # the pair pass that completes the step before a collision
        "pair_wca": step,
        "pair_ref": step,
        "srd_collide": SRD_PARTICLE_B * ns + 32.0 * Cs,
        # preparation passes: their own compulsory traffic
        "bead_pro": 64.0 * nb + 16.0 * nb,
        "filament_pass": 64.0 * nb + 16.0 * nb,
        "scan_cells": 8.0 * C,
        "chunk_sum": 4.0 * C,
        "scatter": 16.0 * nb,
        "stable_gather": 16.0 * nb,
        "srd_hash": 16.0 * (nb + ns) + 8.0 * (nb + ns),
        "srd_scatter": 16.0 * (nb + ns),
        # bead and solvent tables in one launch each
        "srd_scan_cells": 24.0 * Cs,
        "srd_chunk_sum": 8.0 * Cs,
        "advance_step": 8.0,
    }
    return table.get(name, 0.0)


def read_peak():
    try:
        d = json.loads(PEAKS_FILE.read_text())
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


def read_traffic(name: str):
    """DRAM bytes per unit of work of a kernel from the committed ncu summary."""
    try:
        for line in TRAFFIC_FILE.read_text().splitlines():
            parts = line.split()
            if len(parts) >= 3 and parts[0] == name and not line.startswith("#"):
                return float(parts[1]), parts[2]
    except Exception:
        pass
    return None


class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.path = Path(os.environ.get("TMPDIR", "/tmp")) / f"nw_clocks_{os.getpid()}.csv"

    def start(self):
        try:
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=self.fh, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.fh.close()
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.path.read_text().splitlines():
            p = [x.strip() for x in line.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                mx = max(mx, float(p[2]))
            except ValueError:
                continue
            for nm, v in zip(names, p[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        self.path.unlink(missing_ok=True)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def cpu_baseline(cfg, pos, vel, budget_s: float = 20.0):
    """FP64 CPU port of the step (oracle/, OpenMP over all host threads) on a
    bounded sample of the same workload: whole bead steps without SRD plus
    one SRD collision, combined as t_bead + t_srd / gap."""
    sys.path.insert(0, str(REPO / "oracle"))
    import numpy as np

    import oracle as orc

    orc.set_threads(os.cpu_count() or 1)
    nb = cfg.n_beads
    c_beads = cfg.copy()
    c_beads.srd_enabled = 0
    z = np.zeros((nb, 4), np.float64)
    st = dict(pos=pos[:nb], vel=vel[:nb], force=z, force_old=z, tangent=z)
    t0 = time.perf_counter()
    n_bead = 0
    while True:
        st = orc.step(c_beads, st, n_bead, cfg.dt, 64)
        n_bead += 1
        if time.perf_counter() - t0 > budget_s * 0.5 or n_bead >= 20:
            break
    t_bead = (time.perf_counter() - t0) / n_bead
    t_srd = 0.0
    if cfg.srd_enabled:
        t1 = time.perf_counter()
        orc.srd(cfg, pos, vel, nb, cfg.n_solvent, orc.srd_shift(cfg, 0, 64), None, 0, cfg.dt * cfg.srd_gap, 64)
        t_srd = time.perf_counter() - t1
    per_step = t_bead + t_srd / max(1, cfg.srd_gap)
    sample = f"{n_bead} full bead steps ({nb} beads, FP64)" + (
        f" + 1 SRD collision ({nb + cfg.n_solvent} particles), per step = bead + SRD/{cfg.srd_gap}" if cfg.srd_enabled else "")
    return {"value": nb / per_step, "unit": "bead-steps/s", "cores": orc.num_threads(), "kind": "port",
            "sample": sample, "seconds_per_step": per_step}


def workload_config(name: str, seed: int, isolated: bool = False):
    """Configuration and initial state of a single-system workload.  With
    isolated, the configuration is derived in a child process, so that this
    process never loads libnwgb (the reference arm)."""
    from nwgb.init import initial_state

    w = WORKLOADS[name]
    if isolated:
        from nwgb.abi import NwConfig

        code = ("import sys; sys.path.insert(0, %r); from nwgb.init import baseline_config; "
                "sys.stdout.write(bytes(baseline_config(%d, seed=%d)).hex())" % (str(REPO / "nematic-worms_gb300"),
                                                                                w["k"], seed))
        out = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, check=True).stdout
        cfg = NwConfig.from_buffer_copy(bytes.fromhex(out.strip()))
    else:
        from nwgb.init import baseline_config

        cfg = baseline_config(w["k"], seed=seed)
    pos, vel = initial_state(cfg, seed=seed, layout=w["layout"])
    return cfg, pos, vel


def config_block(name, cfg, world):
    return {"workload": name, "filaments": int(cfg.num_filaments), "filament_size": int(cfg.filament_size),
            "beads": cfg.n_beads, "solvent": cfg.n_solvent, "box": [float(cfg.box[0]), float(cfg.box[1])],
            "model": "WCA_WORMS", "srd_gap": int(cfg.srd_gap) if cfg.srd_enabled else None, "dt": float(cfg.dt),
            "global_batch": cfg.n_beads * world, "parallelism": f"replicas x{world}",
            "l2": "state larger than L2 (no flush needed)"}


def job_rate(dist, ms_local: float, units_local: float, device="cpu"):
    """Whole-job throughput over the ranks: the units all ranks processed
    divided by the slowest rank's time (max over ranks).  Returns
    (units per second, max ms)."""
    import torch

    t_ms = torch.tensor([ms_local], dtype=torch.float64, device=device)
    t_units = torch.tensor([units_local], dtype=torch.float64, device=device)
    if dist is not None:
        dist.all_reduce(t_ms, op=dist.ReduceOp.MAX)
        dist.all_reduce(t_units, op=dist.ReduceOp.SUM)
    ms_max = float(t_ms.item())
    return float(t_units.item()) / (ms_max / 1e3), ms_max


def run_reference(args):
    rank, world, _ = env_rank()
    if rank != 0:
        return 0
    import numpy as np

    cfg, pos, vel = workload_config(args.workload, 0, isolated=True)
    sys.path.insert(0, str(REPO / "oracle"))
    import oracle as orc

    orc.set_threads(os.cpu_count() or 1)
    nb = cfg.n_beads
    z = np.zeros((nb, 4), np.float64)
    st = dict(pos=pos.astype(np.float64), vel=vel.astype(np.float64), force=z, force_old=z, tangent=z)
    # each step of this arm is one full step of the workload on the host cores;
    # timed steps cover whole SRD periods (the collision every srd_gap steps
    # is part of the per-step cost) and the run is capped to a few minutes
    period = int(cfg.srd_gap) if cfg.srd_enabled else 1
    t_w = time.perf_counter()
    for s in range(period):
        st = orc.step(cfg, st, s, cfg.dt, 64)
    per_period = max(1e-3, time.perf_counter() - t_w)
    periods = max(1, min(-(-args.steps // period), int(120.0 / per_period)))
    n = periods * period
    t0 = time.perf_counter()
    for s in range(n):
        st = orc.step(cfg, st, period + s, cfg.dt, 64)
    dt = time.perf_counter() - t0
    value = nb * n / dt
    line = {"metric": "bead-steps/s", "value": value, "unit": "bead-steps/s", "n_gpus": world, "steps": n,
            "warmup": period, "ms_per_step": 1e3 * dt / n, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic", "impl": "reference",
            "config": config_block(args.workload, cfg, 1),
            "cpu_baseline": {"value": value, "unit": "bead-steps/s", "cores": orc.num_threads(), "kind": "port",
                             "sample": f"{n} full steps of the workload (FP64 port of the reference step; "
                                       f"{args.steps} requested, capped at ~2 min)"},
            "e2e": {"value": value, "unit": "bead-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def schedule(first_step: int, steps: int, gap: int):
    """Chunks of a K-step run starting at update first_step, aligned to whole
    SRD periods: up to the next period boundary, whole periods, remainder."""
    out = []
    head = (-first_step) % gap
    if head:
        out.append(min(head, steps))
    left = steps - sum(out)
    out += [gap] * (left // gap)
    if left % gap:
        out.append(left % gap)
    return out


def run_steps(sysm, sched, dt):
    launches = 0
    for n in sched:
        sysm.step(n, dt)
        launches += sysm.last_launch_count
    return launches


def warm_and_prepare(sysm, cfg, warmup, steps, chunk):
    """Exactly `warmup` steps, then capture (without running) every graph the
    timed schedule replays.  Returns the schedule."""
    done = 0
    for n in schedule(0, warmup, chunk):
        sysm.step(n, cfg.dt)
        done += n
    sched = schedule(done, steps, chunk)
    at = done
    for n in sched:
        sysm.prepare(n, cfg.dt, at)
        at += n
    sysm.sync()
    return sched


def timed_region(sysm, sched, cfg, stream, dist=None):
    """K steps between a barrier + synchronize on both sides, CUDA events on
    the engine's stream.  Returns (ms, kernel launches)."""
    import torch

    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    launches = run_steps(sysm, sched, cfg.dt)
    ev1.record(stream)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    return ev0.elapsed_time(ev1), launches


def strategies_block(cfg, pos, vel, warmup, steps, stream):
    """The same workload and start under each step strategy: the sorted scheme
    (hash, stable sort and cell bounds every update, as the reference), capped
    per-cell lists, and Verlet lists over those cells (the headline)."""
    import nwgb
    from nwgb import abi

    out = {}
    chunk = GRAPH_STEPS
    for name, strat in (("sorted", abi.NW_STRATEGY_SORTED), ("cell_lists", abi.NW_STRATEGY_CELL_LISTS),
                        ("verlet", abi.NW_STRATEGY_VERLET)):
        c = cfg.copy()
        c.strategy = strat
        with nwgb.System(c) as s:
            s.set_stream(stream.cuda_stream)
            s.set_array(abi.NW_POSITION, pos)
            s.set_array(abi.NW_VELOCITY, vel)
            s.zero_forces()
            sched = warm_and_prepare(s, c, warmup, steps, chunk)
            ms, launches = timed_region(s, sched, c, stream)
            s.sync()
        out[name] = {"ms_per_step": ms / steps, "value": c.n_beads * steps / (ms / 1e3), "steps": steps,
                     "warmup": warmup, "launches_per_step": launches / steps}
    return out


R1 = dict(filaments=20000, filament_size=20, grid=(1024, 1024, 1))


def r1_setters(p, s):
    """main.cpp's setters for the stand-in run (flags -kbT=0.1 -gamma=2
    -kBend=10 -kBond=57 -activity=0.5 -reverse=0 -boundX=0 -boundY=0
    -boundZ=1, hardness at its default = the initial kBond 57.146436) and the
    workload's bond rest length 0.8 (setBondSpringLength)."""
    p.kbT = 0.1
    s.kbT = 0.1
    p.gamma = 2.0
    p.bondBendingK = 10.0
    p.bondSpringK = 57.0
    p.activity = 0.5
    p.reverseProbability = 0.0
    p.spring = 57.146436
    p.bondSpringL = 0.8
    p.boundaryX, p.boundaryY, p.boundaryZ = 0, 0, 1


def ref_dem_r1(warmup, steps, stream):
    """This engine's REF_DEM model (the reference's collideFilaments
    semantics) on the reference-feasible stand-in of the 400k + SRD workload,
    from the reference's reset() state, through the handle API."""
    import nwgb
    from nwgb import abi
    from nwgb.init import reference_reset

    cfg = abi.default_config(abi.NW_MODEL_REF_DEM, R1["filaments"], R1["filament_size"], R1["grid"], True)
    cfg.kT = cfg.srd_kT = 0.1
    cfg.gamma = 2.0
    cfg.bend_k = 10.0
    cfg.bond_k = 57.0
    cfg.activity = 0.5
    cfg.reverse_probability = 0.0
    cfg.spring = 57.146436
    cfg.bond_r0 = 0.8
    cfg.boundary[0], cfg.boundary[1], cfg.boundary[2] = abi.NW_PERIODIC, abi.NW_PERIODIC, abi.NW_WALL
    cfg.dt = 0.005
    pos, vel, tan = reference_reset(cfg)
    with nwgb.System(cfg) as s:
        s.set_stream(stream.cuda_stream)
        s.set_array(abi.NW_POSITION, pos)
        s.set_array(abi.NW_VELOCITY, vel)
        s.set_array(abi.NW_TANGENT, tan)
        s.zero_forces()
        sched = warm_and_prepare(s, cfg, warmup, steps, int(cfg.srd_gap) * 2)
        ms, launches = timed_region(s, sched, cfg, stream)
        s.sync()
    return {"ms_per_step": ms / steps, "value": cfg.n_beads * steps / (ms / 1e3), "steps": steps, "warmup": warmup,
            "beads": cfg.n_beads, "solvent": cfg.n_solvent, "srd_gap": int(cfg.srd_gap), "launches_per_step":
            launches / steps}


def dist_group(world):
    """The NCCL process group of a multi-rank run (None for one rank)."""
    if world <= 1:
        return None
    import torch.distributed as dist

    if not dist.is_initialized():
        dist.init_process_group("nccl", init_method="env://")
    return dist


def run_reference_cuda(args):
    """The reference's own CUDA build (its kernels compiled for sm_103a from its
    source, launched as its C-ABI layer does, thrust sort and cuRAND) running
    its ParticleSystem::update loop on the stand-in configuration: W untimed
    updates, then K updates between CUDA events on the legacy default stream.
    Prints one JSON line; loads no part of this engine."""
    rank, world, _ = env_rank()
    if rank != 0:
        return 0
    sys.path.insert(0, str(REPO / "oracle"))
    import ref_cuda

    why = ref_cuda.available()
    if why:
        print(json.dumps({"impl": "reference_cuda", "unavailable": why}), flush=True)
        return 0
    rs = ref_cuda.RefSystem(reference=(R1["filaments"], R1["filament_size"], R1["grid"], True))
    p, sv = rs.params, rs.solvent
    r1_setters(p, sv)
    rs.reset()
    dt = 0.005
    rs.run(args.warmup, dt)
    ms = rs.run(args.steps, dt)
    nb = rs.n_beads
    line = {"impl": "reference_cuda", "metric": "bead-steps/s", "value": nb * args.steps / (ms / 1e3),
            "unit": "bead-steps/s", "ms_per_step": ms / args.steps, "steps": args.steps, "warmup": args.warmup,
            "config": {"workload": "ref_dem_r1", "beads": nb, "solvent": rs.n_solvent, "grid": list(R1["grid"]),
                       "srd_gap": 5, "dt": dt}}
    rs.close()
    print(json.dumps(line), flush=True)
    return 0


def reference_cuda_block(warmup, steps):
    """Runs the reference CUDA arm in its own process (so that this process
    never loads the reference build) and returns its line."""
    cmd = [sys.executable, str(REPO / "bench.py"), "--impl", "reference_cuda", "--steps", str(steps), "--warmup",
           str(warmup)]
    env = dict(os.environ)
    for k in ("RANK", "WORLD_SIZE", "LOCAL_RANK"):
        env.pop(k, None)
    try:
        r = subprocess.run(cmd, capture_output=True, text=True, timeout=900, env=env)
        for line in r.stdout.splitlines()[::-1]:
            if line.startswith("{"):
                return json.loads(line)
        return {"unavailable": "no output: " + (r.stderr.strip().splitlines() or ["?"])[-1][:300]}
    except Exception as e:  # noqa: BLE001
        return {"unavailable": f"{type(e).__name__}: {e}"[:300]}


def run_ours(args):
    import numpy as np
    import torch

    import nwgb
    from nwgb import abi

    rank, world, local = env_rank()
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", init_method="env://")
    torch.cuda.set_device(local)
    cfg, pos, vel = workload_config(args.workload, seed=rank)
    nb = cfg.n_beads
    sysm = nwgb.System(cfg)
    # the engine runs on a dedicated (non-default) stream that the CUDA events
    # below are recorded on
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    sysm.set_stream(stream.cuda_stream)
    sysm.set_array(abi.NW_POSITION, pos)
    sysm.set_array(abi.NW_VELOCITY, vel)
    sysm.zero_forces()

    chunk = GRAPH_STEPS
    sched = warm_and_prepare(sysm, cfg, args.warmup, args.steps, chunk)
    blob = sysm.checkpoint()
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)  # let the sampler start before the timed region
    reps = []
    gpu_launches = 0
    for r in range(REPEATS):
        if r:
            sysm.restore(blob)  # the same start state for every repeat
            at = sysm.step_index
            for n in sched:
                sysm.prepare(n, cfg.dt, at)
                at += n
            sysm.sync()
        ms_r, gpu_launches = timed_region(sysm, sched, cfg, stream, dist)
        reps.append(ms_r)
    clk = clocks.stop()
    sysm.sync()
    ms = statistics.median(reps)
    value, ms_max = job_rate(dist, ms, nb * args.steps, device="cuda")

    # ---- end to end through the C ABI with host buffers ------------------------------
    e2e_steps = max(chunk, min(200, args.steps))
    hp = torch.empty((nb, 4), dtype=torch.float32, pin_memory=True).numpy()
    hv = torch.empty((nb, 4), dtype=torch.float32, pin_memory=True).numpy()
    hp[:] = sysm.get_array(abi.NW_POSITION, 0, nb)
    hv[:] = sysm.get_array(abi.NW_VELOCITY, 0, nb)

    def e2e_step():
        # inputs from and results to pinned host memory, one synchronisation
        sysm.set_array_async(abi.NW_POSITION, hp, 0)
        sysm.set_array_async(abi.NW_VELOCITY, hv, 0)
        sysm.step(1, cfg.dt)
        sysm.get_array_async(abi.NW_POSITION, hp, 0)
        sysm.get_array_async(abi.NW_VELOCITY, hv, 0)
        sysm.sync()

    for _ in range(GAP):  # one single-step graph per collision phase, built before the clock starts
        e2e_step()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        e2e_step()
    e2e_s = time.perf_counter() - t0
    e2e_value, _ = job_rate(dist, 1e3 * e2e_s, nb * e2e_steps, device="cuda")

    # ---- per-kernel device time (events around every launch) ---------------------------
    prof = sysm.profile(2 * GAP, cfg.dt)
    sysm.sync()
    dom = max((k for k in prof if k != "advance_step"), key=lambda k: prof[k][0])
    dom_ms = prof[dom][0] / prof[dom][1]
    peak, peak_kind = read_peak()
    bytes_launch = alg_bytes(dom, cfg)
    achieved = bytes_launch / (dom_ms / 1e3) / 1e9
    tr = read_traffic(dom)
    traffic = None
    if tr is not None:
        per_unit, unit = tr
        units = {"bead": nb, "particle": nb + cfg.n_solvent, "cell": cfg.n_cells, "srd_cell": cfg.n_srd_cells}.get(unit)
        traffic = per_unit * units if units else None
    total_prof = sum(v[0] for v in prof.values())
    sb = step_bytes(cfg)
    step_gbs = sb / (ms_max / args.steps / 1e3) / 1e9
    roofline = {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "peak_source": f"{peak_kind} hbm_gbs",
                "traffic": traffic, "alg_bytes_per_launch": bytes_launch, "avg_launch_ms": dom_ms,
                "step": {"alg_bytes": sb, "achieved": step_gbs, "frac": step_gbs / peak,
                         "note": "whole step (timed value) against the same peak"},
                "kernel_share": {k: round(v[0] / total_prof, 4) for k, v in sorted(prof.items(), key=lambda kv: -kv[1][0])},
                "kernel_avg_ms": {k: round(v[0] / v[1], 5) for k, v in sorted(prof.items(), key=lambda kv: -kv[1][0])}}
    sysm.close()

    line = None
    if rank == 0:
        line = {"metric": "bead-steps/s", "value": value, "unit": "bead-steps/s", "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_max / args.steps,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
                "data": "synthetic", "config": config_block(args.workload, cfg, world), "clocks": clk,
                "timing": {"repeats": REPEATS, "ms_per_step": [t / args.steps for t in reps],
                           "median_ms_per_step": ms / args.steps, "spread": (max(reps) - min(reps)) / ms,
                           "note": "each repeat restarts from the checkpoint taken after the warm-up"},
                "e2e": {"value": e2e_value, "unit": "bead-steps/s", "h2d_bytes_per_step": nb * 32,
                        "d2h_bytes_per_step": nb * 32, "steps": e2e_steps,
                        "path": "nw_set_array_async(pos, vel) + nw_step(1) + nw_get_array_async(pos, vel) + "
                                "nw_sync per step, pinned host; the host link measures ~200 GB/s per direction"},
                "gpu_launches": gpu_launches, "roofline": roofline}
        if world == 1 and not args.no_extras:
            k_sub = min(args.steps, 1000)
            line["strategies"] = strategies_block(cfg, pos, vel, args.warmup, k_sub, stream)
            if args.workload == "wca_srd_400k":
                k_ref = min(args.steps, 200)
                ours = ref_dem_r1(args.warmup, k_ref, stream)
                theirs = reference_cuda_block(args.warmup, k_ref)
                blk = {"ours_ref_dem": ours, "reference": theirs}
                if "ms_per_step" in theirs:
                    blk["speedup"] = theirs["ms_per_step"] / ours["ms_per_step"]
                line["reference_cuda"] = blk
                line["batch_256"] = batch_block(args, steps=min(args.steps, 1000))
                line["adjoint_64x4k"] = adjoint_block(args)
        if world == 1 and not args.no_cpu_baseline:
            line["cpu_baseline"] = cpu_baseline(cfg, pos.astype(np.float64), vel.astype(np.float64))
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()
    return 0


def run_batch(args):
    line = batch_block(args)
    if env_rank()[0] == 0:
        print(json.dumps(line), flush=True)
    return 0


def batch_block(args, steps=None):
    """Batched replicas: every step of all replicas in one launch, CUDA graphs of
    100 steps, launch shape and neighbour search from the autotuner.  Reported
    beside it: the same replicas run one by one through the single-system step
    (sequential), and one single system holding as many beads (plain)."""
    import math as _m

    import torch

    import nwgb
    from nwgb import abi
    from nwgb.init import batch_configs, initial_state, wca_config

    rank, world, local = env_rank()
    torch.cuda.set_device(local)
    dist = dist_group(world)
    R = WORKLOADS["batch_256"]["batch"]
    cfgs = batch_configs(R, seed=1000)
    states = [initial_state(c, seed=r, layout="rows") for r, c in enumerate(cfgs)]
    if world > 1:
        # one job of R replicas spread over the ranks by bead count
        from nwgb.replicas import partition

        mine = partition([c.n_beads for c in cfgs], world)[rank]
        cfgs, states = [cfgs[r] for r in mine], [states[r] for r in mine]
    total = sum(c.n_beads for c in cfgs)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    chunk = 100
    nchunks = max(1, (args.steps if steps is None else steps) // chunk)

    def timed(step_fn, n):
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        ev0.record(stream)
        for _ in range(n):
            step_fn()
        ev1.record(stream)
        torch.cuda.synchronize()
        return ev0.elapsed_time(ev1)

    b = nwgb.Batch(cfgs)
    b.set_stream(stream.cuda_stream)
    for r, (pos, vel) in enumerate(states):
        b.set_array(r, abi.NW_POSITION, pos)
        b.set_array(r, abi.NW_VELOCITY, vel)
    tune = b.autotune(trial_steps=20)
    warm = 0
    while warm < max(args.warmup, chunk):
        b.step(chunk)
        warm += chunk
    b.sync()
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    ms = timed(lambda: b.step(chunk), nchunks)
    clk = clocks.stop()
    b.sync()
    launches = b.last_launch_count * nchunks
    value, ms = job_rate(dist, ms, total * chunk * nchunks, device="cuda")
    b.close()
    if world > 1:
        line = {"metric": "bead-steps/s", "value": value, "unit": "bead-steps/s", "n_gpus": world,
                "steps": chunk * nchunks, "warmup": warm, "ms_per_step": ms / (chunk * nchunks),
                "higher_is_better": True, "scaling": "strong", "vs_baseline": None, "dtype": "f32",
                "data": "synthetic", "clocks": clk, "gpu_launches": launches,
                "config": {"workload": "batch_256", "replicas": R, "parallelism": f"replicas bin-packed x{world}",
                           "replicas_rank0": len(cfgs), "beads_rank0": total}}
        dist.destroy_process_group()
        return line

    # sequential: the same replicas one by one through the single-system step
    seq_steps = chunk
    seq_ms = 0.0
    for r, c in enumerate(cfgs):
        with nwgb.System(c) as s:
            s.set_stream(stream.cuda_stream)
            s.set_array(abi.NW_POSITION, states[r][0])
            s.set_array(abi.NW_VELOCITY, states[r][1])
            s.step(seq_steps, c.dt)
            seq_ms += timed(lambda: s.step(seq_steps, c.dt), 1)
            s.sync()
    seq_value = total * seq_steps / (seq_ms / 1e3)

    # plain: one system with the same number of beads at the mean packing
    L = 20
    M = int(round(total / L))
    side = _m.sqrt(M * L * _m.pi / 4.0 / 0.45)
    pc = wca_config(M, L, (side, side), activity=1.0, seed=1)
    pp, pv = initial_state(pc, seed=1, layout="rows")
    with nwgb.System(pc) as s:
        s.set_stream(stream.cuda_stream)
        s.set_array(abi.NW_POSITION, pp)
        s.set_array(abi.NW_VELOCITY, pv)
        s.step(chunk, pc.dt)
        s.sync()
        plain_ms = timed(lambda: s.step(chunk, pc.dt), nchunks)
        s.sync()
    plain_value = pc.n_beads * chunk * nchunks / (plain_ms / 1e3)

    line = {"metric": "bead-steps/s", "value": value, "unit": "bead-steps/s", "n_gpus": world,
            "steps": chunk * nchunks, "warmup": warm, "ms_per_step": ms / (chunk * nchunks),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": "batch_256", "replicas": R, "beads": total, "model": "WCA_WORMS",
                       "graph_steps": chunk, "parallelism": f"replicas x{world}",
                       "tuning": {"threads_per_block": tune.threads_per_block, "strategy": int(tune.strategy),
                                  "neighbor_skin": round(float(tune.neighbor_skin), 3),
                                  "cell_capacity": int(tune.cell_capacity),
                                  "autotune_ms_per_step": float(tune.ms_per_step)},
                       "l2": "state larger than L2 (no flush needed)"},
            "clocks": clk, "gpu_launches": launches,
            "sequential": {"value": seq_value, "steps": seq_steps,
                           "path": "each replica alone: nw_step graphs of 100 steps, one after another"},
            "plain": {"value": plain_value, "beads": pc.n_beads, "box": side,
                      "path": "one single system of the same bead count (20-bead worms, packing 0.45)"},
            "batched_over_plain": value / plain_value, "batched_over_sequential": value / seq_value}
    return line


def run_adjoint(args):
    line = adjoint_block(args)
    if env_rank()[0] == 0:
        print(json.dumps(line), flush=True)
    return 0


def adjoint_block(args):
    """Differentiable rollout: forward + adjoint of 200 steps for 64 replicas of
    the 4k-bead workload (FP32), timed on the device; beside it the production
    batched step on the same replicas and steps."""
    import numpy as np
    import torch

    import nwgb
    from nwgb import abi
    from nwgb.adjoint import Rollout, rollout
    from nwgb.init import baseline_config, initial_state
    from nwgb.observables import PairSample, loss_s_cv, velocity_correlation

    from nwgb.replicas import contiguous_block, loss_and_gradient_mean, replica_mean

    rank, world, local = env_rank()
    torch.cuda.set_device(local)
    dist = dist_group(world)
    R_all = WORKLOADS["adjoint_64x4k"]["adjoint"]
    H, SEG = 200, 20
    # this rank's replicas: an equal contiguous block, so that replica r keeps
    # its seed (7 + r), initial state and pair sample on any rank
    mine = contiguous_block(R_all, world, rank)
    R = len(mine)
    cfg = baseline_config(0, seed=7 + mine.start)
    states = [initial_state(cfg, seed=r, layout="patches") for r in mine]
    pos = torch.from_numpy(np.concatenate([s[0] for s in states])).cuda()
    vel = torch.from_numpy(np.concatenate([s[1] for s in states])).cuda()
    ro = Rollout(cfg, R, H, SEG, 32)
    ro.set_state(pos, vel)
    box = [cfg.box[0], cfg.box[1], cfg.box[2]]
    every = PairSample(R_all, cfg.n_beads, 20000, seed=1, device="cuda")
    pairs = PairSample(1, cfg.n_beads, 1, seed=0, device="cuda")
    pairs.i, pairs.j = every.i[mine.start:mine.stop], every.j[mine.start:mine.stop]
    # C_target from a seeded run at the reference parameters (mean over all replicas)
    with torch.no_grad():
        p, v = ro.forward([1.0, 10.0, 57.0, 0.5])
        cv = velocity_correlation(p[:, :3].reshape(R, -1, 3).double(), v[:, :3].reshape(R, -1, 3).double(), pairs,
                                  box)
        target = replica_mean(cv.sum(0), R, dist)[None, :]
    fwd, bwd, red = [], [], []
    reps = max(3, min(10, args.steps // H))
    for k in range(args.warmup + reps):
        th = torch.tensor([1.1, 8.0, 50.0, 0.8], dtype=torch.float64, requires_grad=True)
        p, v = rollout(th, ro)
        L = loss_s_cv(p[:, :3].reshape(R, -1, 3).double(), v[:, :3].reshape(R, -1, 3).double(), cfg.filament_size,
                      box, pairs, target)
        L.backward()
        t0 = time.perf_counter()
        loss, grad = loss_and_gradient_mean(L, th.grad, R, dist)  # one all-reduce of 6 numbers
        t_red = time.perf_counter() - t0
        f_ms, b_ms = ro.timings()
        if k >= args.warmup:
            fwd.append(f_ms)
            bwd.append(b_ms)
            red.append(1e3 * t_red)
    f_ms, b_ms = statistics.median(fwd), statistics.median(bwd)
    ro.close()
    if world > 1:
        job, step_ms = job_rate(dist, f_ms + b_ms + statistics.median(red), R * cfg.n_beads * H, device="cuda")
        line = {"metric": "bead-steps/s", "value": job, "unit": "bead-steps/s", "n_gpus": world, "steps": H * len(fwd),
                "warmup": args.warmup, "ms_per_step": step_ms / H, "higher_is_better": True, "scaling": "strong",
                "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                "config": {"workload": "adjoint_64x4k", "replicas": R_all, "parallelism": f"replica blocks x{world}",
                           "horizon": H, "segment": SEG},
                "adjoint": {"forward_ms": f_ms, "backward_ms": b_ms, "allreduce_ms": statistics.median(red),
                            "loss": float(loss), "grad": [float(x) for x in grad]}}
        dist.destroy_process_group()
        return line
    # production step on the same replicas (batched engine, one launch per step)
    cfgs = [baseline_config(0, seed=7 + r) for r in range(R)]
    stream = torch.cuda.Stream()
    with nwgb.Batch(cfgs) as b:
        b.set_stream(stream.cuda_stream)
        for r, (ps, vs) in enumerate(states):
            b.set_array(r, abi.NW_POSITION, ps)
            b.set_array(r, abi.NW_VELOCITY, vs)
        b.step(H)
        b.sync()
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ev0.record(stream)
        b.step(H)
        ev1.record(stream)
        torch.cuda.synchronize()
        prod_ms = ev0.elapsed_time(ev1)
    nbt = R * cfg.n_beads
    line = {"metric": "bead-steps/s", "value": nbt * H / ((f_ms + b_ms) / 1e3), "unit": "bead-steps/s",
            "n_gpus": world, "steps": H * len(fwd), "warmup": args.warmup, "ms_per_step": (f_ms + b_ms) / H,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": "adjoint_64x4k", "replicas": R, "beads": nbt, "horizon": H, "segment": SEG,
                       "loss": "(S2 - 0.7)^2 + |C_v - C_target|^2, 32 bins"},
            "adjoint": {"forward_ms": f_ms, "backward_ms": b_ms, "backward_over_forward": b_ms / f_ms,
                        "gradient_over_production_step": (f_ms + b_ms) / prod_ms,
                        "production_batched_ms": prod_ms,
                        "note": "forward = the rollout's own frozen-list step (with checkpoints); "
                                "production = the batched engine over the same replicas and steps"}}
    return line


def defect_frame(n_worms, L, box, seed=11):
    """Worms of L beads along a director field with 8 planted +/-1/2 defects."""
    import numpy as np

    rng = np.random.default_rng(seed)
    sites = [(rng.uniform(0.1, 0.9) * box, rng.uniform(0.1, 0.9) * box, q) for q in (0.5, -0.5) * 4]
    m = 0.5 * (L - 1) * 0.8 + 1.0
    c = rng.uniform(m, box - m, (n_worms, 2))
    a = sum(q * np.arctan2(c[:, 1] - y, c[:, 0] - x) for x, y, q in sites) + rng.normal(0, 0.2, n_worms)
    k = np.arange(L) - 0.5 * (L - 1)
    pos = np.zeros((n_worms * L, 4), dtype=np.float32)
    pos[:, 0] = (c[:, None, 0] + 0.8 * k * np.cos(a)[:, None]).ravel()
    pos[:, 1] = (c[:, None, 1] + 0.8 * k * np.sin(a)[:, None]).ravel()
    return pos


def run_defects(args):
    """Defect search (director field + Burgers circuits + clustering) on one
    frame per call, through the public call a user makes (System.find_defects:
    device binning and circuits, host clustering), frames resident on the
    device; the CPU arm is the numpy restatement of the reference's analysis
    on the same frame."""
    import numpy as np
    import torch

    import nwgb
    from nwgb import abi
    from nwgb.init import wca_config

    rank, world, local = env_rank()
    n_worms, L, box, cs = WORKLOADS[args.workload]["defects"]
    pos = defect_frame(n_worms, L, box)
    nb = len(pos)
    steps = min(args.steps, 2000)

    def cpu_time(reps):
        sys.path.insert(0, str(REPO / "oracle"))
        import defects_oracle

        t0 = time.perf_counter()
        for _ in range(reps):
            d = defects_oracle.find_defects(pos[:, :2], L, cs)
        return (time.perf_counter() - t0) / reps, d

    if args.impl == "reference":
        if rank != 0:
            return 0
        for _ in range(min(args.warmup, 1)):
            cpu_time(1)
        per, _ = cpu_time(max(1, min(steps, 5)))
        line = {"metric": "frames/s", "value": 1.0 / per, "unit": "frames/s", "n_gpus": 0, "steps": steps,
                "warmup": args.warmup, "ms_per_step": per * 1e3, "higher_is_better": True, "impl": "reference",
                "config": {"workload": args.workload, "beads": nb, "cell_size": cs},
                "cpu_baseline": {"value": 1.0 / per, "unit": "frames/s", "cores": 1, "kind": "port",
                                 "sample": "the whole frame, numpy restatement of the reference's analysis"},
                "e2e": {"value": 1.0 / per, "unit": "frames/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line), flush=True)
        return 0

    torch.cuda.set_device(local)
    cfg = wca_config(n_worms, L, (box, box), lib=None)
    with nwgb.System(cfg) as s:
        s.set_array(abi.NW_POSITION, pos)
        for _ in range(args.warmup):
            want = s.find_defects(cs)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(steps):
            got = s.find_defects(cs)
        per = (time.perf_counter() - t0) / steps
        # end to end: the frame uploaded from pinned host memory every call
        host = torch.from_numpy(pos).pin_memory().numpy()
        t0 = time.perf_counter()
        for _ in range(steps):
            s.set_array(abi.NW_POSITION, host)
            got = s.find_defects(cs)
        e2e = (time.perf_counter() - t0) / steps
        # the sampling search (analysis/defects.py defaults: 100 points, radius 10)
        sample = np.random.default_rng(3).integers(0, nb, 100)
        for _ in range(3):
            s.sample_defects(sample, 10.0)
        t0 = time.perf_counter()
        for _ in range(20):
            wind = s.sample_defects(sample, 10.0)
        sampling_ms = (time.perf_counter() - t0) / 20 * 1e3
    cpu_per, cpu_d = cpu_time(2) if rank == 0 and not args.no_cpu_baseline else (None, None)
    same = cpu_d is None or (len(cpu_d) == len(got) and np.array_equal(cpu_d["x"], got["x"]))
    line = {"metric": "frames/s", "value": 1.0 / per, "unit": "frames/s", "n_gpus": world, "steps": steps,
            "warmup": args.warmup, "ms_per_step": per * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32/i64", "data": "synthetic",
            "config": {"workload": args.workload, "beads": nb, "cell_size": cs, "defects": int(len(got))},
            "e2e": {"value": 1.0 / e2e, "unit": "frames/s", "h2d_bytes_per_step": int(pos.nbytes),
                    "d2h_bytes_per_step": int(len(got) * 24 + 4)},
            "gpu_launches": steps * 3, "matches_cpu": bool(same), "timing": "host wall clock per synchronous call",
            "sampling": {"points": 100, "radius": 10.0, "ms_per_call": sampling_ms, "kept": int((wind > 0).sum())}}
    if cpu_per is not None:
        line["cpu_baseline"] = {"value": 1.0 / cpu_per, "unit": "frames/s", "cores": 1, "kind": "port",
                                "sample": "the whole frame, numpy restatement of the reference's analysis"}
    if rank == 0:
        print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--gpus", type=int, default=1)
    # the workload is defined as a 10,000-step run: the active drive pumps
    # momentum into the solvent (no Langevin friction with SRD), so the state
    # keeps warming and longer runs measure a different, hotter system
    ap.add_argument("--steps", type=int, default=10000)
    ap.add_argument("--warmup", type=int, default=100)
    ap.add_argument("--impl", choices=["ours", "reference", "reference_cuda"], default="ours")
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default="wca_srd_400k")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-extras", action="store_true", help="skip the strategies / reference_cuda / batch / "
                    "adjoint sub-blocks of the default line")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference_cuda":
        return run_reference_cuda(args)
    if "adjoint" in WORKLOADS[args.workload]:
        if args.impl == "reference":
            print(json.dumps({"impl": "reference", "unavailable": "the reference has no gradients"}), flush=True)
            return 0
        return run_adjoint(args)
    if "defects" in WORKLOADS[args.workload]:
        return run_defects(args)
    if "batch" in WORKLOADS[args.workload]:
        if args.impl == "reference":
            print(json.dumps({"impl": "reference", "unavailable": "the reference has no batched replicas; "
                              "its arm runs the single-system workloads"}), flush=True)
            return 0
        return run_batch(args)
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
