"""The oracle (CPU restatement, oracle/ppf_oracle.c) against the golden
vectors the reference program itself produced (tests/golden/), and against a
freshly compiled reference where its sources are present."""
import os

import numpy as np
import pytest

import oracle
import oracle.build_ref as build_ref
from helpers import golden_cases, golden_dt, load_golden, smooth_state

# bit-exact on x86-64 gcc -O2 (no FMA contraction); arm64 gcc contracts
# a*b+c into FMAs by default, which moves results by a few ulp
TOL = 1e-12


@pytest.mark.parametrize("name", golden_cases())
def test_oracle_matches_reference_output(name):
    d, meta = load_golden(name)
    p = oracle.reference_params(dt=golden_dt(meta))
    etaS, etaL, c = d["in_etaS"], d["in_etaL"], d["in_c"]
    if not meta["fix_etaL"]:
        etaL = np.ones_like(etaL)   # the reference's /etaL read is a no-op (phasefield.c:1032)
    saves = d["saves"]
    done = 0
    state = (etaS, etaL, c)
    last_eta_sums = None
    for k, row in enumerate(saves):
        it = int(row[0])
        nsteps = it + 1 - done       # save at iteration `it` follows it+1 sweeps
        s0, s1, s2, sums = oracle.run(*state, nsteps, bc=meta["bc"], params=p,
                                      n_iter_init=meta["n_iter_init"] - done)
        if meta["n_iter_init"] - done <= 0:
            # c-only segment: detaS/detaL keep the last full step's values
            # (sweep_fields_c never writes them, phasefield.c:406-476)
            sums[1:] = last_eta_sums
        last_eta_sums = sums[1:].copy()
        done += nsteps
        state = (s0, s1, s2)
        for f, arr in zip(("etaS", "etaL", "c"), state):
            ref = d[f"out{k + 1}_{f}"]
            assert np.abs(arr - ref).max() <= TOL, (name, k, f, np.abs(arr - ref).max())
        # the convergence line prints the sums with 5 significant digits
        np.testing.assert_allclose(sums, row[1:4], rtol=6e-5, atol=1e-300)
        np.testing.assert_allclose(np.sqrt(sums[0]), row[4], rtol=6e-5)


def test_oracle_conserves_solute_periodic_and_noflux():
    st = smooth_state((10, 9, 8), seed=3)
    m0 = st[2].sum()
    for bc in (0, 1):
        _, _, c, _ = oracle.run(*st, 50, bc=bc)
        assert abs(c.sum() - m0) <= 1e-12 * abs(m0)


@pytest.mark.skipif(not os.path.exists(build_ref.REF_SRC), reason="reference sources absent")
@pytest.mark.parametrize("bc", [0, 1])
def test_oracle_matches_fresh_reference_build(bc, tmp_path):
    br = build_ref
    from oracle import read_fields, write_fields
    shape = (7, 9, 11)
    st = smooth_state(shape, seed=11 + bc)
    inp = str(tmp_path / "x.h5")
    write_fields(inp, *st)
    exe = br.build(*shape, bc=bc, n_iter=13, n_save=12)
    r = br.run(exe, inp)
    assert r["rc"] == 0, r["stderr"]
    out = read_fields(str(tmp_path / "x_1.h5"))
    mine = oracle.run(*st, 13, bc=bc)
    for a, b in zip(out, mine[:3]):
        assert np.abs(a - b).max() <= TOL


def test_derive_matches_reference_constants():
    d = oracle.derive()
    assert d["dt"] == 0.125 / 1e-14
    assert d["m"] == 6.0 * 2.0 / 7.0
    assert d["kappa"] == 3 * 0.25 * 2.0 * 7.0
    ML = 1e-14 / 1e9
    assert d["L"] == 4.0 / 3.0 * d["m"] / d["kappa"] * (0.5 * (0.0 + ML) / ((0.999 - 0.476) ** 2))
