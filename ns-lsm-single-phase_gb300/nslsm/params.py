"""Level-set parameters (the `global_lsm` module of the reference) and the
reader of the reference's positional deck `ind3dmg_LSM.dat`.

`LsmParams` mirrors `struct lsm_params` (include/lsm_c.h) field by field;
`read_ind3dmg_lsm` follows the record sequence of `init_input_fileLSM`
(src/init_LSM.F90:129-183), including `delti_lsm = delti / numiter_lsm`.
"""
from __future__ import annotations

import dataclasses as dc
import re
from typing import List, Sequence

from ._lib import LsmParams as _CParams


@dc.dataclass
class LsmParams:
    epslsm: float = 0.0
    numiter_lsm: int = 1
    delti_lsm: float = 0.0
    RNitermax: int = 15
    RNtimestep: float = 0.00078125
    RNfreq: int = 1
    btype_lsm: Sequence[int] = (1, 1, 1, 1, 1, 1)
    bc_extrapolation_order: int = 1
    isnarrow: int = 0
    narrowcoef: float = 3.0
    orderAD: int = 1
    sussman_correction_method: int = 0
    call_levelsetmethod: bool = True
    call_reinitialisation: bool = True
    hybrid_reinitialisation: bool = False
    TotalVolumeComputation: bool = True
    GlobalMassCorrection: bool = False
    BigPhi: float = 5.0
    epsReinitialisation: float = 1.0e-5
    M_Sphi0: int = 1
    reinit_scheme: int = 0              # 1: reinitialisation_test2, the reference's live call
    write_global_volume: bool = False
    OrderReinitialisationBoundaries: int = 1
    ENOBCReinitialisation: bool = False
    ConvergenceToleranceGeomReini: float = 1.0e-9

    def to_c(self) -> _CParams:
        p = _CParams()
        for f in dc.fields(self):
            v = getattr(self, f.name)
            if f.name == "btype_lsm":
                for i in range(6):
                    p.btype_lsm[i] = int(v[i])
            elif isinstance(v, bool):
                setattr(p, f.name, int(v))
            else:
                setattr(p, f.name, v)
        return p

    def replace(self, **kw) -> "LsmParams":
        return dc.replace(self, **kw)


# --------------------------------------------------------------- deck reader
def _tokens(line: str) -> List[str]:
    line = line.split("!")[0]
    out = []
    for t in re.split(r"[,\s]+", line.strip()):
        if not t:
            continue
        m = re.fullmatch(r"(\d+)\*(.+)", t)
        if m:
            out.extend([m.group(2)] * int(m.group(1)))
        else:
            out.append(t)
    return out


def _real(t: str) -> float:
    return float(t.lower().replace("d", "e"))


def _logical(t: str) -> bool:
    s = t.strip().lower().lstrip(".")
    if s.startswith("t"):
        return True
    if s.startswith("f"):
        return False
    raise ValueError(f"not a Fortran logical: {t!r}")


class _ListDirected:
    """Fortran list-directed READ: each statement starts a new record, may
    continue on following lines, and discards what is left of its last line."""

    def __init__(self, text: str):
        self.lines = text.splitlines()
        self.pos = 0

    def read(self, n: int) -> List[str]:
        vals: List[str] = []
        while len(vals) < n:
            if self.pos >= len(self.lines):
                raise ValueError("end of file while reading ind3dmg_LSM.dat")
            vals.extend(_tokens(self.lines[self.pos]))
            self.pos += 1
        return vals[:n]


def read_ind3dmg_lsm(path_or_text: str, delti: float, nzone: int = 1, myzone: int = 1) -> LsmParams:
    """Parse an `ind3dmg_LSM.dat` deck (src/init_LSM.F90:134-169)."""
    try:
        with open(path_or_text) as f:
            text = f.read()
    except (OSError, ValueError):
        text = path_or_text
    r = _ListDirected(text)
    p = LsmParams()
    eps, niter = r.read(2)
    p.epslsm, p.numiter_lsm = _real(eps), int(niter)
    r.read(1)          # thetainc
    r.read(4)          # drho, dmu, diss_w, diss_a
    r.read(2)          # FrLSM, WeLSM
    r.read(4)          # IG, IGitermax, IGtimestep, IGstep2
    a, b, c = r.read(3)
    p.RNitermax, p.RNtimestep, p.RNfreq = int(a), _real(b), int(c)
    r.read(1)          # phi_outputiter
    r.read(1)          # k_surface
    bt = [int(t) for t in r.read(6 * nzone)]
    p.btype_lsm = tuple(bt[6 * (myzone - 1): 6 * myzone])
    p.bc_extrapolation_order = int(r.read(1)[0])
    a, b = r.read(2)
    p.isnarrow, p.narrowcoef = int(a), _real(b)
    p.orderAD = int(r.read(1)[0])
    r.read(1)          # nobstacles
    p.sussman_correction_method = int(r.read(1)[0])
    p.call_levelsetmethod = _logical(r.read(1)[0])
    p.call_reinitialisation = _logical(r.read(1)[0])
    p.hybrid_reinitialisation = _logical(r.read(1)[0])
    r.read(1)          # sweep_lsqm
    r.read(1)          # radius_lsqm
    p.ConvergenceToleranceGeomReini = _real(r.read(1)[0])
    p.TotalVolumeComputation = _logical(r.read(1)[0])
    p.GlobalMassCorrection = _logical(r.read(1)[0])
    nsave = int(r.read(1)[0])
    if nsave > 0:
        r.read(nsave)  # save_LSdebug_tsteps
    p.epsReinitialisation = _real(r.read(1)[0])
    r.read(1)          # OrderLSAdvectionBoundaries
    p.OrderReinitialisationBoundaries = int(r.read(1)[0])
    p.ENOBCReinitialisation = _logical(r.read(1)[0])
    p.BigPhi = _real(r.read(1)[0])
    p.delti_lsm = delti / float(p.numiter_lsm)
    return p
