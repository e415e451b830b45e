"""Search parameters: the gParams fields on the DSLIM path.

Mirrors ``gParams`` (source/core/include/slm_dsts.h:359-418) and the way the
reference's parameter parser fills it (source/app/hicops.cpp:494-688).
"""
from __future__ import annotations

import dataclasses

import numpy as np


@dataclasses.dataclass
class gParams:
    """Field names and meanings of the reference's gParams.

    ``dF`` is in bins: the reference stores (uint)(tolerance_Da * scale), with
    the default scale of 100 (hicops.cpp:564 reads dF before scale). ``dM`` is
    in Da. ``mods`` is a list of (residues, mass_Da, max_per_peptide) and
    ``vmods_per_pep`` the overall limit per peptide.
    """
    min_len: int = 6
    max_len: int = 40
    maxz: int = 3
    topmatches: int = 10
    scale: int = 100
    min_shp: int = 4
    min_cpsm: int = 4
    min_mass: int = 500
    max_mass: int = 5000
    dF: int = 1
    dM: float = 500.0
    res: float = 0.01
    expect_max: float = 20.0
    base_int: int = 100000
    min_int: int = 1000
    threads: int = 8
    spadmem: int = 2000000000
    vmods_per_pep: int = 0
    mods: list = dataclasses.field(default_factory=list)

    def mod_mass_scaled(self, i: int) -> int:
        """(uint)(atof(mass) * scale), as hicops.cpp:661 stores it."""
        return int(np.floor(np.float64(self.mods[i][1]) * np.float64(self.scale)))

    @property
    def nlen(self) -> int:
        return self.max_len - self.min_len + 1

    def write_ref_params(self, path: str) -> None:
        """Key/value file read by the oracle's reference driver."""
        with open(path, "w") as f:
            for k in ("threads", "min_len", "max_len", "maxz", "topmatches", "scale",
                      "min_shp", "min_cpsm", "spadmem", "min_mass", "max_mass", "dF",
                      "base_int", "min_int", "vmods_per_pep"):
                f.write(f"{k} {getattr(self, k)}\n")
            f.write(f"dM {self.dM!r}\nres {self.res!r}\nexpect_max {self.expect_max!r}\n")
            for res, mass, per in self.mods:
                f.write(f"mod {res} {mass!r} {per}\n")


def parse_uparams(path: str) -> gParams:
    """Read a reference ``uparams.txt`` (fixed line order, hicops.cpp:494-688).

    Quirks kept: dF is converted with the default scale (100) because the
    file gives dF before scale; base_int is multiplied by 1000; min_int is a
    ratio of base_int; the mod mass is scaled after scale is known.
    """
    with open(path) as f:
        lines = [ln.rstrip("\n") for ln in f]
    it = iter(lines)
    nxt = lambda: next(it)
    p = gParams()
    for _ in range(3):           # dbpath, datapath, workspace
        nxt()
    p.threads = int(nxt())
    nxt()                        # maxprepthds
    p.min_len = int(nxt())
    p.max_len = int(nxt())
    p.maxz = int(nxt())
    p.dF = int(np.floor(float(nxt()) * 100))   # params.scale still holds its default here
    p.dM = float(nxt())
    p.res = float(nxt())
    p.scale = int(nxt())
    p.min_mass = int(nxt())
    p.max_mass = int(nxt())
    p.topmatches = int(nxt())
    p.expect_max = float(nxt())
    p.min_shp = int(nxt())
    p.min_cpsm = int(nxt())
    p.base_int = int(nxt()) * 1000
    p.min_int = int(float(nxt()) * float(p.base_int))
    p.spadmem = int(nxt()) * 1024 * 1024
    nxt()                        # distribution policy
    nvars = int(nxt())
    if nvars > 0:
        p.vmods_per_pep = int(nxt())
        for _ in range(nvars):
            res = nxt().upper()[:4]
            mass = float(nxt())
            per = int(nxt())
            p.mods.append((res, mass, per))
    return p
