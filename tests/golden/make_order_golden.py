"""Generate tests/golden/order_2d.npz: tangents and order parameters the
reference's own analysis code gives on seeded synthetic worm frames.

Runs, from the reference checkout given by --reference (read only),
analysis/afa/utils.py compute_tangents and the function
compute_relative_orientations of analysis/analyze_correlations.py (taken
from the file's source: the module itself imports plotting packages that
are not installed here) on a frame built with analysis/afa/data.py Frame.
The sample indices the function draws with np.random.randint are drawn again
with the same seed and stored with the results.

usage: python tests/golden/make_order_golden.py --reference <checkout>
"""
from __future__ import annotations

import argparse
import ast
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent


def worm_frame(rng, box, n_worms, L, bond, angle_fn, jitter):
    """n_worms straight worms of L beads (float32), centres uniform in the box,
    directions angle_fn(centre) + Gaussian jitter."""
    c = rng.uniform(0.0, box, size=(n_worms, 2))
    a = angle_fn(c[:, 0], c[:, 1]) + rng.normal(0.0, jitter, n_worms)
    k = np.arange(L) - 0.5 * (L - 1)
    x = c[:, None, 0] + bond * k[None, :] * np.cos(a)[:, None]
    y = c[:, None, 1] + bond * k[None, :] * np.sin(a)[:, None]
    out = np.zeros((n_worms * L, 3), dtype=np.float32)
    out[:, 0] = x.ravel()
    out[:, 1] = y.ravel()
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", required=True)
    args = ap.parse_args()
    ref = Path(args.reference) / "analysis"
    sys.path.insert(0, str(ref))
    from afa.data import Frame  # the reference's frame class
    from afa.utils import compute_tangents

    src = (ref / "analyze_correlations.py").read_text()
    tree = ast.parse(src)
    fn = next(n for n in tree.body if isinstance(n, ast.FunctionDef) and n.name == "compute_relative_orientations")
    ns = {"np": np, "Frame": Frame}
    exec(compile(ast.Module(body=[fn], type_ignores=[]), "analyze_correlations.py", "exec"), ns)
    cro = ns["compute_relative_orientations"]

    rng = np.random.default_rng(2024)
    frames = {
        "nematic": (200, 10, 60.0, lambda x, y: np.zeros_like(x), 0.15),
        "isotropic": (200, 10, 60.0, lambda x, y: rng.uniform(0, 2 * np.pi, x.shape), 0.0),
        "polar": (150, 12, 50.0, lambda x, y: 0.6 + 0.0 * x, 0.3),
        "swirl": (300, 8, 70.0, lambda x, y: np.arctan2(y - 35.0, x - 35.0) + np.pi / 2, 0.1),
    }
    out = {}
    for k, (name, (n, L, box, fn_a, jit)) in enumerate(frames.items()):
        r = worm_frame(rng, box, n, L, 0.8, fn_a, jit)
        frame = Frame(r, np.zeros(len(r)), L)
        t_ref = compute_tangents(r, L)
        n_samples = 5000
        np.random.seed(100 + k)
        dist, nn, tt, S, P = cro(frame, n_samples, [box, box, 0.0])
        np.random.seed(100 + k)
        i, j = np.random.randint(0, len(frame), size=[2, n_samples])
        out.update({f"{name}_r": r, f"{name}_L": np.int64(L), f"{name}_box": np.array([box, box, 0.0]),
                    f"{name}_t": t_ref, f"{name}_i": i, f"{name}_j": j, f"{name}_dist": dist, f"{name}_nn": nn,
                    f"{name}_tt": tt, f"{name}_S": np.float64(S.real), f"{name}_P": np.float64(P)})
    out["names"] = np.array(list(frames))
    np.savez_compressed(HERE / "order_2d.npz", **out)
    print("wrote", HERE / "order_2d.npz")


if __name__ == "__main__":
    main()
