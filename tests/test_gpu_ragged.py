"""GPU parity on a synthetic cluster with ragged cells (1 to 20 membranes),
random gap-junction partners and boundary membranes (tests/synthetic.py),
against the NumPy oracle. BETSE's Voronoi clusters stay at 8 membranes or
fewer per cell, so the long-cell paths of the segment sums and of the tile
partition are covered only here."""
import numpy as np
import pytest

import golden_io as gi
import oracle
import synthetic

pytestmark = pytest.mark.gpu

N = 30


def _engine(d, precision):
    from betse_gb300.engine import ClusterEngine
    cg, sp, Dm, st, _ = gi.engine_inputs(d)
    eng = ClusterEngine(cg, sp, precision)
    eng.set_membrane_diffusivity(Dm)
    eng.upload(**st)
    return eng


@pytest.fixture(scope='module')
def ragged():
    d = synthetic.ragged_fixture()
    g, p, s = gi.geometry(d), gi.params(d), gi.state(d)
    out = oracle.run(g, p, s, N, outputs_last=True)
    return d, s, out


def test_ragged_fp64_state_and_outputs(ragged):
    d, ref, ref_out = ragged
    with _engine(d, 'fp64') as eng:
        eng.step(N, outputs=True)
        eng.check_stable()
        s = eng.download()
        o = eng.outputs()
    ok, err, bound = gi.vm_err_ok(d, s['vm'], ref.vm, ref.cc_cells)
    assert ok, (err, bound)
    for k in ('cc_cells', 'cc_at_mem'):
        assert gi.rel_err(s[k], getattr(ref, k)) < 1e-10, k
    assert gi.rel_err(s['cc_env'], ref.cc_env[:, 0]) < 1e-10
    floors = gi.output_floors(d, ref.cc_cells, o)
    for k in ('fluxes_mem', 'fluxes_gj', 'rate_NaKATP', 'rho_cells', 'Jn', 'I_mem', 'J_cell_x', 'J_cell_y',
              'vm_ave', 'dvm', 'E_gj_x', 'E_gj_y'):
        r = np.asarray(ref_out[k])
        err = np.max(np.abs(o[k] - r))
        assert err <= 1e-10 * np.max(np.abs(r)) + floors.get(k, 0.0), (k, err)


def test_ragged_split_state(ragged):
    d, ref, _ = ragged
    with _engine(d, 'split') as eng:
        eng.step(N)
        eng.check_stable()
        s = eng.download()
    assert np.max(np.abs(s['vm'] - ref.vm)) < 1e-6
    assert gi.rel_err(s['cc_cells'], ref.cc_cells) < 1e-5


@pytest.mark.parametrize('tpb', [192, 256])
def test_ragged_persistent_equals_tile_kernel(tpb):
    d = synthetic.ragged_fixture()
    res = []
    for persist in (False, True):
        with _engine(d, 'split') as e:
            e.set_launch_config(tpb, persist)
            e.step(40)
            res.append(e.download())
    for k in res[0]:
        assert np.array_equal(res[0][k], res[1][k]), k


@pytest.mark.parametrize('precision', ['fp64', 'split'])
def test_ragged_in_a_batch_equals_alone(precision):
    from betse_gb300.engine import BatchEngine, ClusterEngine
    ds = [synthetic.ragged_fixture(), gi.load('noecm_r50_s7'), synthetic.ragged_fixture(seed=11, n_cells=30)]
    ins = [gi.engine_inputs(d) for d in ds]
    with BatchEngine([x[0] for x in ins], [x[1] for x in ins], precision) as b:
        b.set_membrane_diffusivity([x[2] for x in ins])
        b.upload_states([x[3] for x in ins])
        b.step(25)
        got = b.download_states()
    for (cg, sp, Dm, st, _), s in zip(ins, got):
        with ClusterEngine(cg, sp, precision) as e:
            e.set_membrane_diffusivity(Dm)
            e.upload(**st)
            e.step(25)
            ref = e.download()
        for k in ('vm', 'cc_cells', 'cc_at_mem', 'cc_env'):
            assert np.array_equal(s[k], ref[k]), k
