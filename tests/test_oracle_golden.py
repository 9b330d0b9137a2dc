"""The CPU oracle against the golden vectors produced by the reference's own
CPU code (src/Main/reg.avx.cpp, pot.avx.cpp) and by the oracle itself."""
import numpy as np
import pytest

from conftest import load_golden, rel_vec_err, rows_equal, unpack_list
from oracle import oracle as O

CASES = ["plummer2048_equal", "mflag_plummer512", "overflow_plummer512", "ragged_n37"]


def run_oracle(g):
    return O.regf_fp64(g["m"], g["x"], g["v"], g["h2"], g["dtr"], g["x"][g["ii"]],
                       g["v"][g["ii"]], int(g["lmax"]), int(g["nnbmax"]), int(g["m_flag"]))


@pytest.mark.parametrize("name", CASES)
def test_oracle_reproduces_its_golden(name):
    g = load_golden(name)
    acc, jrk, pot, lst = run_oracle(g)
    lmax = int(g["lmax"])
    assert rows_equal(lst, unpack_list(g["fp64_cnt"], g["fp64_ids"], lmax)) == []
    np.testing.assert_allclose(acc, g["fp64_acc"], rtol=1e-12, atol=1e-14)
    np.testing.assert_allclose(jrk, g["fp64_jrk"], rtol=1e-12, atol=1e-14)
    np.testing.assert_allclose(pot, g["fp64_pot"], rtol=1e-12)


@pytest.mark.parametrize("name", CASES)
def test_oracle_matches_reference_cpu_path(name):
    """Same neighbour sets and counts (incl. overflow flags) as reg.avx.cpp;
    forces within the reference's own FP32 error (measured <= 1.2e-6)."""
    g = load_golden(name)
    acc, jrk, pot, lst = run_oracle(g)
    lmax = int(g["lmax"])
    assert rows_equal(lst, unpack_list(g["ref_cnt"], g["ref_ids"], lmax)) == []
    ok = lst[:, 0] >= 0
    assert rel_vec_err(g["ref_acc"][ok], acc[ok]).max() < 2e-5
    assert np.percentile(rel_vec_err(g["ref_acc"][ok], acc[ok]), 99) < 5e-6
    assert rel_vec_err(g["ref_jrk"][ok], jrk[ok]).max() < 2e-4
    assert (np.abs(g["ref_pot"][ok] - pot[ok]) / pot[ok]).max() < 1e-5


def test_port_matches_reference_cpu_path():
    g = load_golden("plummer2048_equal")
    p = O.Port()
    p.send(g["m"], g["x"], g["v"])
    acc, jrk, pot, lst = p.regf(g["h2"], g["dtr"], g["x"], g["v"], int(g["lmax"]),
                                int(g["nnbmax"]))
    assert rows_equal(lst, unpack_list(g["ref_cnt"], g["ref_ids"], int(g["lmax"]))) == []
    assert rel_vec_err(acc, g["ref_acc"]).max() < 5e-6
    assert (np.abs(pot - g["ref_pot"]) / g["ref_pot"]).max() < 5e-6


def test_pot_oracle_golden():
    g = load_golden("pot_plummer2048")
    all_ = O.pot_fp64(g["m"], g["x"])
    np.testing.assert_allclose(all_, g["fp64_all"], rtol=1e-13)
    assert (np.abs(all_ - g["ref_all"]) / all_).max() < 1e-6
    sub = O.pot_fp64(g["m"], g["x"], int(g["istart"]), int(g["ni"]))
    np.testing.assert_allclose(sub, g["fp64_sub"], rtol=1e-13)
    assert (np.abs(sub - g["ref_sub"]) / sub).max() < 1e-6
    port = O.Port.pot(g["m"], g["x"])
    assert (np.abs(port - g["ref_all"]) / all_).max() < 1e-6


def test_oracle_contract_details():
    """self listed, strict '<', neighbours excluded from force and potential,
    ascending lists, overflow -> -count"""
    m = np.array([0.5, 0.25, 0.25])
    x = np.array([[0.0, 0, 0], [1.0, 0, 0], [0, 2.0, 0]])
    v = np.zeros((3, 3))
    # h2 exactly 1.0: body 1 at r2 == 1 is NOT a neighbour (strict)
    acc, jrk, pot, lst = O.regf_fp64(m, x, v, [1.0], [0.0], x[:1], v[:1], 4, 3)
    assert list(lst[0, :2]) == [1, 0]
    np.testing.assert_allclose(pot[0], 0.25 / 1.0 + 0.25 / 2.0)
    np.testing.assert_allclose(acc[0], [0.25, 0.25 / 4.0, 0.0])
    acc, jrk, pot, lst = O.regf_fp64(m, x, v, [4.5], [0.0], x[:1], v[:1], 4, 3)
    assert list(lst[0, :4]) == [3, 0, 1, 2]
    assert pot[0] == 0.0 and np.all(acc[0] == 0.0)
    acc, jrk, pot, lst = O.regf_fp64(m, x, v, [4.5], [0.0], x[:1], v[:1], 4, 2)
    assert lst[0, 0] == -3
    # predicted-distance criterion: body 1 moving onto body 0 within dtr
    v2 = v.copy(); v2[1] = [-1.0, 0, 0]
    _, _, _, lst = O.regf_fp64(m, x, v2, [0.25], [0.9], x[:1], v[:1], 4, 3)
    assert list(lst[0, :3]) == [2, 0, 1]
