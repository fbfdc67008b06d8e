"""The `ind3dmg_LSM.dat` reader follows init_input_fileLSM's record order
(src/init_LSM.F90:134-169) with Fortran list-directed semantics."""
import pytest

from nslsm import LsmParams
from nslsm.params import read_ind3dmg_lsm

DECK = """\
0.0234375 2          ! epslsm, numiter_lsm
0.0
1.0e-3, 1.0e-2, 1.0, 0.1
0.5 1.0
0 10 0.001 1
15 0.00078125 1      ! RNitermax, RNtimestep, RNfreq
100
40
1 1 1 1 0 2
1
1, 3.0d0
1
0
0
.true.
.true.
.false.
3
2.5
1.0e-4
T
.false.
2
46 47
1.0E-05
2
1
.false.
5.0
.false.
.false.
"""


def test_reads_every_record():
    p = read_ind3dmg_lsm(DECK, delti=0.01)
    assert p.epslsm == 0.0234375 and p.numiter_lsm == 2
    assert p.delti_lsm == 0.01 / 2
    assert (p.RNitermax, p.RNtimestep, p.RNfreq) == (15, 0.00078125, 1)
    assert tuple(p.btype_lsm) == (1, 1, 1, 1, 0, 2)
    assert p.isnarrow == 1 and p.narrowcoef == 3.0
    assert p.orderAD == 1 and p.sussman_correction_method == 0
    assert p.call_levelsetmethod and p.call_reinitialisation and not p.hybrid_reinitialisation
    assert p.TotalVolumeComputation and not p.GlobalMassCorrection
    assert p.epsReinitialisation == 1e-5 and p.BigPhi == 5.0
    assert p.ConvergenceToleranceGeomReini == 1.0e-4


def test_hybrid_deck_selects_the_geometric_branch():
    deck = DECK.replace(".true.\n.true.\n.false.\n3\n2.5\n1.0e-4\nT\n.false.",
                        ".true.\n.true.\n.true.\n3\n2.5\n1.0E-09\nT\n.true.")
    p = read_ind3dmg_lsm(deck, delti=0.01)
    assert p.hybrid_reinitialisation and p.GlobalMassCorrection
    assert p.ConvergenceToleranceGeomReini == 1.0e-9
    c = p.to_c()
    assert c.hybrid_reinitialisation == 1 and c.GlobalMassCorrection == 1 and c.ConvergenceToleranceGeomReini == 1e-9


def test_multi_zone_btype_and_repeat_counts():
    deck = DECK.replace("1 1 1 1 0 2", "6*1\n2 2 2 2 2 2")
    p = read_ind3dmg_lsm(deck, delti=0.02, nzone=2, myzone=2)
    assert tuple(p.btype_lsm) == (2,) * 6


def test_truncated_deck_raises():
    with pytest.raises(ValueError):
        read_ind3dmg_lsm("0.1 1\n0.0\n", delti=1.0)


def test_params_to_c_roundtrip():
    p = LsmParams(epslsm=0.3, btype_lsm=(0, 1, 2, 0, 1, 2), call_reinitialisation=False)
    c = p.to_c()
    assert c.epslsm == 0.3 and list(c.btype_lsm) == [0, 1, 2, 0, 1, 2] and c.call_reinitialisation == 0
