"""Trajectory frames in the reference's text format.

Writer: include/nwgb.h nw_writer_* (snapshot on the device, copy and
formatting off the step loop).  read_frames: the frame layout read by the
reference's analysis code (analysis/afa/io.py:4-25): a particle count line,
a comment line (here the JSON parameter object), then one line per particle
"label x y z vx vy vz" (A = bead, B = solvent)."""
from __future__ import annotations

import ctypes as C
import json
from pathlib import Path
from typing import Iterator

import numpy as np

from .abi import check


class Writer:
    """Appends frames of a System to a file; close (or use as a context
    manager) before the System is closed."""

    def __init__(self, system, path, append: bool = False):
        self.lib = system.lib
        self._h = C.c_void_p()
        check(self.lib.nw_writer_open(system._h, str(path).encode(), 1 if append else 0, C.byref(self._h)),
              "nw_writer_open")

    def frame(self, iteration: int, dt: float) -> None:
        check(self.lib.nw_writer_frame(self._h, int(iteration), float(dt)), "nw_writer_frame")

    def flush(self) -> None:
        check(self.lib.nw_writer_flush(self._h), "nw_writer_flush")

    def close(self) -> None:
        if self._h:
            h, self._h = self._h, C.c_void_p()
            check(self.lib.nw_writer_close(h), "nw_writer_close")

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def read_frames(path) -> Iterator[dict]:
    """Frames of a trajectory file: dict(header=parsed JSON, labels (n,),
    pos (n, 3), vel (n, 3))."""
    with open(Path(path)) as fp:
        while True:
            line = fp.readline()
            if not line:
                return
            n = int(line)
            header = json.loads(fp.readline())
            labels = np.empty(n, dtype="<U1")
            data = np.empty((n, 6))
            for i in range(n):
                parts = fp.readline().split()
                labels[i] = parts[0]
                data[i] = [float(x) for x in parts[1:7]]
            yield dict(header=header, labels=labels, pos=data[:, :3], vel=data[:, 3:])
