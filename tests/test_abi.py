"""The C-ABI boundary without a GPU: the library loads, exports every symbol
the headers declare, agrees with the Python binding's struct layout, and the
reference's own host code links against it unchanged."""
from __future__ import annotations

import ctypes as C
import re
import shutil
import subprocess
from pathlib import Path

import pytest

from conftest import REPO
from nwgb import abi

def _reference():
    from nwgb.build import reference_tree

    return reference_tree() or Path("/nonexistent")


REFERENCE = _reference()


def declared_functions(header: Path):
    text = header.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"^\s*(?:nw_status|void|int|uint32_t|uint64_t|size_t|const char\*)\s+(\w+)\s*\(", text, flags=re.M)
    return sorted(set(names))


@pytest.mark.parametrize("header", ["nwgb.h", "nw_legacy.h", "nwgb_batch.h", "nwgb_adjoint.h"])
def test_library_exports_every_declared_symbol(lib, header):
    names = declared_functions(REPO / "include" / header)
    assert len(names) >= {"nw_legacy.h": 20, "nwgb.h": 25, "nwgb_batch.h": 15, "nwgb_adjoint.h": 7}[header]
    out = subprocess.run(["nm", "-D", "--defined-only", str(abi.LIB_PATH)], capture_output=True, text=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if " T " in line}
    missing = [n for n in names if n not in exported]
    assert not missing, missing
    for n in names:
        assert hasattr(lib, n)


def test_reference_legacy_symbol_set_is_complete(lib):
    # the 20 extern "C" functions of the reference's launch layer (+ cudaInit's siblings)
    ref = ["cudaInit", "randomizeUniform", "randomizeGaussian", "allocateArray", "freeArray", "threadSync",
           "copyArrayFromDevice", "copyArrayToDevice", "setParameters", "setSolventParameters",
           "integrateFilaments", "integrateSolvent", "calcHash", "reorderDataAndFindCellStart",
           "collideFilaments", "collideSolvent", "filamentForces", "sortParticles", "reverseFilaments",
           "langevinThermostat", "solventCellCentorOfMomentum", "solventIsokineticThermostat"]
    for n in ref:
        assert hasattr(lib, n), n


def test_struct_layout_and_version(lib):
    assert lib.nw_abi_version() == abi.NW_ABI_VERSION
    assert lib.nw_config_size() == C.sizeof(abi.NwConfig)


def test_config_defaults_and_validation(lib):
    c = abi.default_config(abi.NW_MODEL_REF_DEM, 6000, 35, (1024, 128, 1), False, lib)
    # reference constructor defaults (simulation/particleSystem.cpp:64-105)
    assert c.radius == 0.5 and c.cell_size[0] == 1.0 and c.box[0] == 1024.0 and c.origin[0] == -512.0
    assert c.bond_r0 == pytest.approx(0.4) and c.bend_k == pytest.approx(0.001) and c.gamma == pytest.approx(0.01)
    assert c.hash_mode == abi.NW_HASH_MASK
    assert lib.nw_config_validate(C.byref(c)) == abi.NW_OK
    s = abi.default_config(abi.NW_MODEL_REF_DEM, 10, 10, (64, 64, 1), True, lib)
    assert tuple(s.srd_grid) == (32, 32, 1) and s.srd_cell_size[0] == 2.0 and s.num_solvent == 10 * 32 * 32
    assert s.srd_gap == 5 and s.srd_alpha == pytest.approx(2.26893)
    bad = c.copy()
    bad.grid[0] = 100  # the power-of-two mask needs power-of-two grids
    abi.check(lib.nw_config_finalize(C.byref(bad)))
    assert lib.nw_config_validate(C.byref(bad)) == abi.NW_ERR_INVALID
    w = abi.default_config(abi.NW_MODEL_WCA_WORMS, 400, 10, (89, 89, 1), False, lib)
    assert w.dim == 2 and w.noise_dt_scaling == 1 and w.hash_mode == abi.NW_HASH_MODULO
    assert lib.nw_config_validate(C.byref(w)) == abi.NW_OK
    small = w.copy()
    small.cell_size[0] = 1.0  # below the cut-off: the 3x3 stencil would miss pairs
    abi.check(lib.nw_config_finalize(C.byref(small)))
    assert lib.nw_config_validate(C.byref(small)) == abi.NW_ERR_INVALID
    for k in ("filament_size",):
        z = w.copy()
        setattr(z, k, 0)
        assert lib.nw_config_validate(C.byref(z)) == abi.NW_ERR_INVALID
    v = w.copy()
    v.abi_version = 99
    assert lib.nw_config_validate(C.byref(v)) == abi.NW_ERR_INVALID


def test_status_strings(lib):
    assert lib.nw_status_string(abi.NW_OK) == b"ok"
    assert b"non-finite" in lib.nw_status_string(abi.NW_ERR_NONFINITE)


@pytest.mark.skipif(not (REFERENCE / "simulation" / "particleSystem.cpp").exists() or shutil.which("g++") is None,
                    reason="needs the reference tree")
def test_reference_host_code_links_against_libnwgb(tmp_path):
    """The reference's unchanged main.cpp + particleSystem.cpp link against
    libnwgb.so in place of particleSystem_cuda.cu (drop-in at the C ABI)."""
    sim, common = REFERENCE / "simulation", REFERENCE / "common"
    exe = tmp_path / "nw_dropin"
    cmd = ["g++", "-std=c++17", "-O1", "-w", f"-I{sim}", f"-I{common}", "-I/usr/local/cuda/include",
           str(sim / "main.cpp"), str(sim / "particleSystem.cpp"), "-o", str(exe),
           f"-L{abi.LIB_DIR}", "-lnwgb", f"-Wl,-rpath,{abi.LIB_DIR}", "-L/usr/local/cuda/lib64", "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    assert exe.exists()


def declared_arities(header: Path):
    """{function name: number of parameters} of the header's prototypes."""
    text = re.sub(r"/\*.*?\*/", "", header.read_text(), flags=re.S)
    text = re.sub(r"//[^\n]*", "", text)
    out = {}
    for name, params in re.findall(
            r"^\s*(?:nw_status|void|int|uint32_t|uint64_t|size_t|const char\*)\s+(\w+)\s*\(([^;{]*?)\)\s*;",
            text, flags=re.M | re.S):
        p = " ".join(params.split())
        out[name] = 0 if p in ("", "void") else p.count(",") + 1
    return out


@pytest.mark.parametrize("header", ["nwgb.h", "nw_legacy.h", "nwgb_batch.h", "nwgb_adjoint.h"])
def test_python_binding_matches_every_prototype(header):
    """Every function the ctypes binding declares has the header prototype's
    number of parameters (a drifted signature would pass garbage)."""
    declared = declared_arities(REPO / "include" / header)
    bound = {name: len(args) for name, _, args in abi.HANDLE_API + abi.LEGACY_API + abi.BATCH_API + abi.ADJOINT_API}
    checked = 0
    for name, n in declared.items():
        if name in bound:
            assert bound[name] == n, (name, bound[name], n)
            checked += 1
    assert checked >= {"nw_legacy.h": 18, "nwgb.h": 25, "nwgb_batch.h": 12, "nwgb_adjoint.h": 6}[header], checked
