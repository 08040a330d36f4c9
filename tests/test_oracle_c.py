"""The C restatement of the step (``oracle/c/bx_oracle.c``, the multi-threaded
CPU baseline) against BETSE's golden states and the NumPy oracle, with and
without extracellular spaces.  CPU only."""
import numpy as np
import pytest

import golden_io as gi

CASES = list(gi.CASES)


@pytest.fixture(scope='module')
def cstep():
    from oracle import cstep as cs
    try:
        cs.build()
    except Exception as e:      # no compiler: the C baseline is optional for the CPU suite
        pytest.skip(f'gcc/OpenMP unavailable: {e}')
    return cs


@pytest.mark.parametrize('name', CASES)
def test_c_restatement_matches_betse(cstep, name):
    d = gi.load(name)
    g, p, s = gi.geometry(d), gi.params(d), gi.state(d)
    st = cstep.Stepper(g, p, s)
    done = 0
    for cp in d['meta_checkpoints']:
        st.step(int(cp) - done)
        done = int(cp)
        got = st.state()
        ok, err, bound = gi.vm_err_ok(d, got['vm'], d[f's{cp}_vm'], d[f's{cp}_cc_cells'])
        assert ok, (cp, err, bound)
        assert gi.rel_err(got['cc_cells'], d[f's{cp}_cc_cells']) < 1e-10
        assert gi.rel_err(got['cc_at_mem'], d[f's{cp}_cc_at_mem']) < 1e-10
        assert gi.rel_err(got['cc_env'], d[f's{cp}_cc_env']) < 1e-10
        if 'gjopen' in got:
            assert gi.rel_err(got['gjopen'], d[f's{cp}_gjopen']) < 1e-10


@pytest.mark.parametrize('name', ['noecm_r50_s7', 'ecm_r40_s5_sharp'])
def test_c_restatement_matches_numpy_oracle(cstep, name):
    import oracle
    d = gi.load(name)
    g, p, s = gi.geometry(d), gi.params(d), gi.state(d)
    st = cstep.Stepper(g, p, s)
    st.step(25)
    oracle.run(g, p, s, 25)
    got = st.state()
    for k in ('cc_cells', 'cc_at_mem', 'cc_env'):
        assert gi.rel_err(got[k], np.asarray(getattr(s, k)).reshape(got[k].shape)) < 1e-12, k
    ok, err, bound = gi.vm_err_ok(d, got['vm'], s.vm, s.cc_cells, rel=1e-12)
    assert ok, (err, bound)
    if bool(p.is_ecm):
        for k in ('E_env_x', 'E_env_y'):
            assert gi.rel_err(got[k], getattr(s, k)) < 1e-9, k


def test_c_restatement_thread_count_independent(cstep):
    d = gi.load('noecm_r80_s1')
    out = []
    for threads in (1, 3):
        st = cstep.Stepper(gi.geometry(d), gi.params(d), gi.state(d), threads=threads)
        st.step(50)
        out.append(st.state())
    for k in out[0]:
        assert np.array_equal(out[0][k], out[1][k]), k


@pytest.mark.parametrize('name', ['noecm_r50_s7', 'ecm_r50_s3'])
def test_c_restatement_with_a_boundary_potential(cstep, name):
    """An applied boundary potential (sim.Phi_b) shifts vm and, with ECM,
    v_env: the C restatement follows the NumPy oracle."""
    import oracle
    d = gi.load(name)
    g, p, s = gi.geometry(d), gi.params(d), gi.state(d)
    rng = np.random.default_rng(8)
    s.Phi_b = rng.uniform(-2e-3, 2e-3, size=s.Phi_b.shape)
    st = cstep.Stepper(g, p, s)
    st.step(10)
    oracle.run(g, p, s, 10)
    got = st.state()
    for k in ('cc_cells', 'cc_env'):
        assert gi.rel_err(got[k], np.asarray(getattr(s, k)).reshape(got[k].shape)) < 1e-12, k
    ok, err, bound = gi.vm_err_ok(d, got['vm'], s.vm, s.cc_cells, rel=1e-12)
    assert ok, (err, bound)


def test_c_restatement_on_ragged_cells(cstep):
    """Cells of 1 to 20 membranes and random partners (tests/synthetic.py)."""
    import oracle
    import synthetic
    d = synthetic.ragged_fixture()
    g, p, s = gi.geometry(d), gi.params(d), gi.state(d)
    st = cstep.Stepper(g, p, s)
    st.step(30)
    oracle.run(g, p, s, 30)
    got = st.state()
    for k in ('cc_cells', 'cc_at_mem', 'cc_env'):
        assert gi.rel_err(got[k], getattr(s, k)) < 1e-12, k
    ok, err, bound = gi.vm_err_ok(d, got['vm'], s.vm, s.cc_cells, rel=1e-12)
    assert ok, (err, bound)
