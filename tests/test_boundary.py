"""The C-ABI boundary without a GPU: the library loads, exports every symbol
``include/bx.h`` declares, and rejects inconsistent geometry before touching
the device; the host records reproduce BETSE's index maps bit-exactly."""
import ctypes as ct
import os
import re

import numpy as np
import pytest

import golden_io as gi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared_symbols():
    src = open(os.path.join(ROOT, 'include', 'bx.h')).read()
    src = re.sub(r'/\*.*?\*/', '', src, flags=re.S)
    return sorted(set(re.findall(r'\b(bx_[a-z0-9_]+)\s*\(', src)))


@pytest.fixture(scope='module')
def lib():
    from betse_gb300 import build, _lib
    build.build()
    return _lib.load()


def test_library_exports_every_declared_symbol(lib):
    from betse_gb300 import _lib
    names = _declared_symbols()
    assert len(names) >= 15
    for n in names:
        assert hasattr(lib, n), n
        assert n in _lib.SIGNATURES, n
    assert lib.bx_abi_version() == 1


def test_struct_layouts_match_header(lib):
    from betse_gb300 import _lib
    # bx_params: 4 int32 + 29 doubles + 4 arrays of 8 doubles + gating (2 int32 + 2 doubles)
    assert ct.sizeof(_lib.BxParams) == 16 + 8 * 29 + 4 * 8 * 8 + 8 + 16 + 24 + 8
    assert ct.sizeof(_lib.BxGeom) == 16 + 8 * 14 + 16 + 8
    assert ct.sizeof(_lib.BxStepStatus) == 8 + 4 + 4 + 8 + 4 + 4


def _geom(d):
    cg, sp, Dm, st, _ = gi.engine_inputs(d)
    return cg, sp


@pytest.mark.parametrize('name', gi.CASES)
def test_csr_reproduces_cells_index_maps(name):
    d = gi.load(name)
    cg, _ = _geom(d)
    m2c = d['geom_mem_to_cells']
    assert np.array_equal(np.repeat(np.arange(cg.n_cells), np.diff(cg.cell_mem_ptr)), m2c)
    assert np.array_equal(cg.mem_to_cells, m2c)
    assert np.array_equal(cg.nn_i, d['geom_nn_i'])
    assert np.array_equal(np.nonzero(cg.bflag)[0], np.sort(d['geom_bflags_mems']))
    assert np.array_equal(np.diff(cg.cell_mem_ptr), d['geom_num_mems'])
    # BETSE's nn_i is an involution on paired membranes
    nn = cg.nn_i
    assert np.array_equal(nn[nn], np.arange(cg.n_mems))


def _expect_einval(lib, cg, sp):
    from betse_gb300 import _lib
    g, p = cg.to_c(), sp.to_c()
    h = ct.c_void_p()
    rc = lib.bx_cluster_create(ct.byref(g), ct.byref(p), 0, ct.byref(h))
    assert rc == _lib.BX_EINVAL, rc
    assert not h.value
    return lib.bx_last_error().decode()


def test_create_rejects_bad_geometry(lib):
    d = gi.load('noecm_r20_s2')
    cg, sp = _geom(d)
    bad = cg.nn_i.copy()
    bad[3] = cg.n_mems + 5
    cg2 = cg.__class__(**{**cg.__dict__, 'nn_i': bad})
    assert 'nn_i' in _expect_einval(lib, cg2, sp)
    ptr = cg.cell_mem_ptr.copy()
    ptr[-1] += 1
    cg3 = cg.__class__(**{**cg.__dict__, 'cell_mem_ptr': ptr})
    assert 'cell_mem_ptr' in _expect_einval(lib, cg3, sp)
    mp = cg.map_mem2ecm.copy()
    mp[0] = -1
    cg4 = cg.__class__(**{**cg.__dict__, 'map_mem2ecm': mp})
    assert 'map_mem2ecm' in _expect_einval(lib, cg4, sp)
    sp2 = sp.replace(iK=sp.iNa)
    assert 'iNa' in _expect_einval(lib, cg, sp2)


def test_fp64_probe_rejects_bad_arguments(lib):
    from betse_gb300 import _lib
    assert lib.bx_fp64_fma_probe(0, 10, 1.0, 1.0, ct.c_void_p(16), None) == _lib.BX_EINVAL
    assert lib.bx_fp64_fma_probe(4, 0, 1.0, 1.0, ct.c_void_p(16), None) == _lib.BX_EINVAL
    assert lib.bx_fp64_fma_probe(4, 10, 1.0, 1.0, None, None) == _lib.BX_EINVAL
    assert lib.bx_fp64_fma_probe((1 << 22) + 1, 10, 1.0, 1.0, ct.c_void_p(16), None) == _lib.BX_EINVAL
    assert b'bad arguments' in lib.bx_last_error()


def test_geometry_rejects_noncontiguous_cells():
    from betse_gb300.cluster import ClusterGeometry
    d = gi.load('noecm_r20_s2')
    g = gi.geometry(d)
    m2c = g.mem_to_cells.copy()
    m2c[[0, -1]] = m2c[[-1, 0]]
    g.mem_to_cells = m2c
    with pytest.raises(ValueError):
        ClusterGeometry.from_cells(g)


def test_engine_missing_library_fails_loudly(tmp_path):
    from betse_gb300 import _lib
    with pytest.raises(_lib.BxLibraryError):
        _lib._lib_backup = _lib._lib
        try:
            _lib._lib = None
            _lib.load(str(tmp_path / 'nope.so'))
        finally:
            _lib._lib = _lib._lib_backup


def test_ctypes_layouts_match_c_compiler(tmp_path):
    """Compile a probe against include/bx.h and compare struct sizes/offsets."""
    import shutil
    import subprocess
    from betse_gb300 import _lib
    cc = shutil.which('gcc') or shutil.which('cc')
    if cc is None:
        pytest.skip('no C compiler')
    src = tmp_path / 'probe.c'
    src.write_text('#include <stdio.h>\n#include <stddef.h>\n#include "bx.h"\n'
                   'int main(void){printf("%zu %zu %zu %zu %zu %zu %zu\\n",'
                   'sizeof(bx_geom), sizeof(bx_params), sizeof(bx_state), sizeof(bx_outputs),'
                   'sizeof(bx_step_status), offsetof(bx_params, zs), offsetof(bx_geom, gj_len));'
                   'printf("%zu %zu %zu %zu %zu %zu\\n", sizeof(bx_net_term), sizeof(bx_net_substance),'
                   'sizeof(bx_net_reaction), sizeof(bx_net_spec), offsetof(bx_net_substance, growth_mod),'
                   'offsetof(bx_net_reaction, keq));return 0;}\n')
    exe = tmp_path / 'probe'
    subprocess.run([cc, '-I', os.path.join(ROOT, 'include'), str(src), '-o', str(exe)], check=True)
    got = [int(x) for x in subprocess.run([str(exe)], capture_output=True, text=True,
                                          check=True).stdout.split()]
    want = [ct.sizeof(_lib.BxGeom), ct.sizeof(_lib.BxParams), ct.sizeof(_lib.BxState),
            ct.sizeof(_lib.BxOutputs), ct.sizeof(_lib.BxStepStatus),
            _lib.BxParams.zs.offset, _lib.BxGeom.gj_len.offset,
            ct.sizeof(_lib.BxNetTerm), ct.sizeof(_lib.BxNetSubstance), ct.sizeof(_lib.BxNetReaction),
            ct.sizeof(_lib.BxNetSpec), _lib.BxNetSubstance.growth_mod.offset, _lib.BxNetReaction.keq.offset]
    assert got == want
