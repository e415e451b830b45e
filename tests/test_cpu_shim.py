"""CPU test of the reference-side binding (hicops_gb300/shim/hicops_dslim_shim.cpp):
compiled against the reference's own headers (dslim.h:49,184, dslim_fileout.h:29,
slm_dsts.h) with its layout assertions (pepEntry = hc_entry, Queries arrays,
SLM_varAA residues), linked with libhicops_gb300.so and run. Skipped where the
reference sources are not mounted (they never are on the GPU machine)."""
import os
import shutil
import subprocess

import pytest

from hicops_gb300 import build as B
from oracle import refrun

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HC_ERR_NO_DEVICE = -3022
ERR_INVLD_PTR = -3008


def test_shim_compiles_against_the_reference_and_links(tmp_path):
    import torch
    ref = refrun.reference_dir()
    if not os.path.isdir(os.path.join(ref, "source", "core", "include")):
        pytest.skip("reference sources not mounted")
    if shutil.which("g++") is None:
        pytest.skip("no g++")
    assert refrun.build(ref)  # also writes the reference's generated config.hpp / common.hpp
    lib = B.build(quiet=True)
    exe = str(tmp_path / "shim_test")
    cmd = ["g++", "-std=c++17", "-O1", "-fopenmp", "-DUSE_OMP", "-w",
           "-I", os.path.join(ROOT, "oracle", "_ref", "gen"), "-I", os.path.join(ref, "source", "core", "include"),
           "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "hicops_gb300", "shim", "hicops_dslim_shim.cpp"),
           os.path.join(ROOT, "tests", "shim", "shim_main.cpp"),
           "-L", os.path.dirname(lib), "-lhicops_gb300", f"-Wl,-rpath,{os.path.dirname(lib)}", "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr[-2000:]
    out = dict(zip(r.stdout.split()[0::2], map(int, r.stdout.split()[1::2])))
    if torch.cuda.is_available():
        assert out["construct"] == 0 and out["query"] == 0
    else:
        # the reference's status_t carries the library's code: no device here
        assert out["construct"] == HC_ERR_NO_DEVICE
        assert out["query"] == ERR_INVLD_PTR  # no context was created
    assert out["deinit"] == 0
