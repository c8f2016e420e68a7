"""The reference's RNG-dependent test goldens, pinned on the oracle.

test/test_system.jl and test/test_updaters.jl start from `fieldinit!(sys; scale = 0.1,
seed = 12345)`, i.e. Julia's seeded `randn` stream.  oracle/julia_rng.py restates that stream
(dSFMT-19937 MersenneTwister, ziggurat randn, Dict order), the fixture
tests/golden/julia_seed_fields.npz holds its output, and the FP64 oracle evaluated on those
fields must give the numbers the reference's tests assert.
"""
import math

import numpy as np
import pytest

import julia_rng as J
import pf_oracle as O
import reference_values as RV
from polyfields import workloads as W


def test_mersenne_twister_matches_julias_documented_draws():
    """Julia's manual: `Random.seed!(1234); rand()` (the `seed!` docstring) and
    `randn(MersenneTwister(1234), ComplexF64)` = 0.6133070881429037 - 0.6376291670853887im,
    i.e. two randn draws scaled by 1/sqrt(2)."""
    rng = J.MersenneTwister(1234)
    assert rng.rand() == 0.5908446386657102
    pytest.importorskip("mpmath")
    rng = J.MersenneTwister(1234)
    re, im = J.randn(rng), J.randn(rng)
    assert re == 0.8673472019512456
    assert im == -0.9017438158568171
    assert re / math.sqrt(2) == pytest.approx(0.6133070881429037, rel=1e-15)
    assert im / math.sqrt(2) == pytest.approx(-0.6376291670853887, rel=1e-15)


def test_dict_iteration_order_of_monomer_ids():
    assert J.dict_order([1, 2, 3]) == [2, 3, 1]
    assert J.dict_order([1, 2]) == [2, 1]
    assert J.dict_order([3, 1, 2]) == [2, 3, 1]   # insertion order does not matter without collisions


def test_fixture_is_what_the_restatement_draws():
    pytest.importorskip("mpmath")
    import make_julia_seed_fields as MK
    fresh = MK.fields()
    d = np.load(f"{W.GOLDEN}/julia_seed_fields.npz")
    assert sorted(d.files) == sorted(fresh)
    for k in d.files:
        assert np.array_equal(d[k], fresh[k]), k


def test_oracle_reproduces_test_system_goldens():
    """test/test_system.jl:29-34 (`@test ... ≈ ...`, rtol sqrt(eps)); the oracle matches to a
    few ulps."""
    sys, point, chain = W.reference_test_system(O)
    point.density_update()
    chain.density_update()
    g = RV.TEST_SYSTEM
    assert point.Q == pytest.approx(g["point_Q"], rel=1e-14)
    assert chain.Q == pytest.approx(g["chain_Q"], rel=1e-14)
    assert sys.free_energy() == pytest.approx(g["free_energy"], rel=1e-14)
    assert sys.free_energy_bulk() == pytest.approx(g["free_energy_bulk"], rel=1e-14)
    assert sys.scfstress()[0] == pytest.approx(g["scfstress_1"], rel=1e-14)


def test_oracle_reproduces_test_updaters_goldens():
    """test/test_updaters.jl:18-30: Euler, NAG and Anderson updaters set up on one system,
    then 10 steps of each in turn.  Euler and NAG to a few ulps; Anderson within the
    reference test's own tolerance (its Gram solve amplifies last-bit FFT differences)."""
    sys = W.reference_test_updaters_system(O)
    u1 = O.EulerUpdater(method="PECE", lam=0.005)
    u1.setup(sys)
    u2 = O.MomentumUpdater(method="NAG", lam=0.005)
    u2.setup(sys)
    u3 = O.AndersonUpdater(nhist=5)
    u3.setup(sys)
    g = RV.TEST_UPDATERS
    for _ in range(10):
        u1.step()
    assert sys.free_energy() == pytest.approx(g["after_euler"], rel=1e-14)
    for _ in range(10):
        u2.step()
    assert sys.free_energy() == pytest.approx(g["after_nag_commented_out"], rel=1e-14)
    for _ in range(10):
        u3.step()
    assert sys.free_energy() == pytest.approx(g["after_anderson"], rel=1e-9)
    assert sys.free_energy() == pytest.approx(g["after_anderson"], rel=math.sqrt(np.finfo(float).eps))


def test_oracle_replays_the_notebooks_seeded_momentum_run():
    """examples/examples.ipynb cells 11-12 from the seed: every line scft! printed (the state
    after k updates, formatted as the reference formats it; quirk Q5: inside the loop ferr and
    fhelm come from the residuals of the pre-update field, simulate.jl:92-107), the convergence
    step and the returned SCFTResults.  About 20 s: 3273 MomentumUpdater steps of the 256-point blend."""
    run = RV.NOTEBOOK_BLEND_RUN
    sys = W.notebook_blend_seeded_system(O)
    sys.residuals_update()  # scft! starts with residuals!(sys) (simulate.jl:66)
    state = {0: (sys.field_error(), sys.free_energy())}
    r = O.scft(sys, O.MomentumUpdater(method="MOM", lam=0.01),
               opts=O.SCFTOptions(nsteps=5000, nsout=0, ftol=1e-5, stol=5e-5))
    for step, ferr, fhelm in r.history:
        state[step + 1] = (ferr, fhelm)
    for k, (ferr, fhelm) in run["printed"].items():
        assert f"{state[k][0]:8e}" == f"{ferr:8e}", k
        assert f"{state[k][1]:.5e}" == f"{fhelm:.5e}", k
    ferr, fhelm = run["converged_line"]  # "Converged @ step = n": the state after n + 1 updates
    assert f"{state[run['nsteps'] + 1][0]:8e}" == f"{ferr:8e}"
    assert f"{state[run['nsteps'] + 1][1]:.5e}" == f"{fhelm:.5e}"
    assert r.converged and r.nsteps == run["nsteps"]
    assert r.ferr == pytest.approx(RV.BLEND_FINAL["ferr"], rel=1e-9)
    assert r.fhelm == pytest.approx(RV.BLEND_FINAL["fhelm"], rel=1e-13)


# ----------------------------------------------------------------------------- the package's stream
def test_package_fieldinit_stream_gives_the_fixture():
    """polyfields.julia_random (what pf.fieldinit(sys; seed, scale) draws) writes exactly the
    fields of the fixture, i.e. the reference's fieldinit! fields for its tests and notebook."""
    from polyfields import julia_random as JR
    d = np.load(f"{W.GOLDEN}/julia_seed_fields.npz")
    for name, mids, shape, scale in (("system", (1, 2, 3), (1, 1, 32), 0.1), ("updaters", (1, 2), (1, 1, 32), 0.1),
                                     ("nbblend", (1, 2, 3), (1, 1, 256), 0.05)):
        got = JR.fieldinit_fields(mids, shape, seed=12345, scale=scale)
        assert sorted(got) == sorted(mids)
        for mid in mids:
            assert np.array_equal(got[mid], d[f"{name}_w{mid}"]), (name, mid)


@pytest.mark.parametrize("seed", [12345, 1234, 0, 2 ** 40 + 7])
def test_package_stream_matches_the_oracle_restatement(seed):
    """The package's vectorised generator against the oracle's word-by-word one, bit for bit:
    scalar draws, the cache path (< 384 elements), the direct block fill (>= 384) and the
    ziggurat's rejection draws."""
    pytest.importorskip("mpmath")
    from polyfields import julia_random as JR
    a, b = J.MersenneTwister(seed), JR.MersenneTwister(seed)
    for n in (5, 13, 32, 256, 383, 384, 385, 1003, 5000, 7):
        assert np.array_equal(np.array(J.randn_array(a, n)), b.randn_array(n)), n
    assert a.rand() == b.rand()


def test_package_ziggurat_tables_are_the_oracles():
    pytest.importorskip("mpmath")
    from polyfields import julia_random as JR
    k, w, f = JR._zig()
    ko, wo, fo = J._tables()
    assert [int(x) for x in k] == list(ko)
    assert np.array_equal(w, np.array(wo)) and np.array_equal(f, np.array(fo))


def test_negative_seed_continues_the_stream():
    """fieldinit!(sys; seed = -1) does not reseed (src/fileio.jl:15-17): a second call continues
    the process-wide stream."""
    from polyfields import julia_random as JR
    first = JR.fieldinit_fields((1, 2), (1, 4, 8), seed=7, scale=1.0)
    second = JR.fieldinit_fields((1, 2), (1, 4, 8), seed=-1, scale=1.0)
    rng = JR.MersenneTwister(7)
    expect = [rng.randn_array(32) for _ in range(4)]   # Dict order (2, 1), then again
    assert np.array_equal(first[2].ravel(), expect[0]) and np.array_equal(first[1].ravel(), expect[1])
    assert np.array_equal(second[2].ravel(), expect[2]) and np.array_equal(second[1].ravel(), expect[3])


def test_dict_order_beyond_the_first_resize():
    """Eleven or more monomer ids: the table grows (64 slots for 11 keys); the package and
    the oracle model it alike, and the order of up to 10 keys is unchanged by the growth rule."""
    from polyfields import julia_random as JR
    rng = np.random.default_rng(3)
    for n in (1, 3, 10, 11, 12, 25, 40):
        keys = [int(k) for k in rng.choice(1000, size=n, replace=False)]
        got = JR.dict_order(keys)
        assert got == J.dict_order(keys) and sorted(got) == sorted(keys), n
    assert JR.dict_order([1, 2, 3]) == [2, 3, 1]
