"""ctypes binding of libbx.so (declarations mirror ``include/bx.h``).

The library is the only compute path: if it is missing or fails to load, every
entry point raises ``BxLibraryError`` -- there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as ct
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, 'libbx.so')

MAX_IONS = 8
BX_OK = 0
BX_EINVAL = -22
BX_ENOMEM = -12
BX_ECUDA = -5
BX_EUNSTABLE = -1001
BX_ESTATE = -1002
PLAIN_FP64 = 0
SPLIT_FP32 = 1

_dp = ct.POINTER(ct.c_double)
_ip = ct.POINTER(ct.c_int32)
_fp = ct.POINTER(ct.c_float)
_u8p = ct.POINTER(ct.c_uint8)


class BxLibraryError(RuntimeError):
    """libbx.so is missing, failed to load or a call failed."""


class BxGeom(ct.Structure):
    _fields_ = [('n_cells', ct.c_int32), ('n_mems', ct.c_int32),
                ('grid_ny', ct.c_int32), ('grid_nx', ct.c_int32),
                ('cell_mem_ptr', _ip), ('nn_i', _ip), ('bflag', _u8p),
                ('map_mem2ecm', _ip), ('mem_sa', _dp), ('mem_nx', _dp),
                ('mem_ny', _dp), ('gj_weight', _dp),
                ('smooth_weight_mem', _dp), ('smooth_weight_o', _dp),
                ('cell_vol', _dp), ('cell_sa', _dp), ('diviterm', _dp),
                ('mem_sa_per_env', _dp), ('gj_len', ct.c_double),
                ('delta', ct.c_double), ('R_rads', _dp)]


class BxParams(ct.Structure):
    _fields_ = [('n_ions', ct.c_int32), ('iNa', ct.c_int32), ('iK', ct.c_int32),
                ('is_ecm', ct.c_int32)] + \
        [(n, ct.c_double) for n in (
            'F', 'R', 'T', 'dt', 'cm', 'tm', 'gj_surface', 'gj_block',
            'nakatp_block', 'alpha_NaK', 'KmNK_Na', 'KmNK_K', 'KmNK_ATP', 'cATP',
            'cADP', 'cPi', 'deltaGATP', 'vol_env', 'cell_height', 'q', 'kb', 'eo',
            'er', 'sharpness', 'cell_radius', 'true_cell_size', 'ko_env', 'sigma',
            'mu')] + \
        [('zs', ct.c_double * MAX_IONS), ('D_free', ct.c_double * MAX_IONS),
         ('D_gj', ct.c_double * MAX_IONS), ('c_env_bound', ct.c_double * MAX_IONS),
         ('v_sensitive_gj', ct.c_int32), ('iCa', ct.c_int32), ('gj_vthresh', ct.c_double),
         ('gj_min', ct.c_double), ('alpha_Ca', ct.c_double), ('KmCa_Ca', ct.c_double),
         ('KmCa_ATP', ct.c_double), ('cell_polarizability', ct.c_double)]


NET_MAX_SUBSTANCES = 16
NET_MAX_REACTIONS = 32
NET_MAX_TERMS = 256
NET_MAX_STOICH = 4
TERM_ACT, TERM_ACT_INDEP, TERM_INH, TERM_DIRECT_POS, TERM_DIRECT_NEG = 0, 1, 2, 3, 4


class BxNetTerm(ct.Structure):
    _fields_ = [('kind', ct.c_int32), ('substance', ct.c_int32), ('env_zone', ct.c_int32),
                ('pad', ct.c_int32), ('Km', ct.c_double), ('n', ct.c_double)]


class BxNetSubstance(ct.Structure):
    _fields_ = [(n, ct.c_double) for n in ('z', 'Dm', 'Do', 'Dgj', 'time_factor', 'r_production',
                                          'r_decay', 'decay_max', 'gad_scale_factor')] + \
        [(n, ct.c_int32) for n in ('growth', 'update_intra', 'gj_impermeable', 'growth_term0',
                                   'growth_nterm', 'decay_term0', 'decay_nterm', 'pad')] + \
        [('growth_mod', _dp), ('growth_target', _u8p)]


class BxNetReaction(ct.Structure):
    _fields_ = [('n_reactants', ct.c_int32), ('n_products', ct.c_int32),
                ('reactant', ct.c_int32 * NET_MAX_STOICH), ('product', ct.c_int32 * NET_MAX_STOICH),
                ('reactant_coeff', ct.c_double * NET_MAX_STOICH), ('reactant_Km', ct.c_double * NET_MAX_STOICH),
                ('product_coeff', ct.c_double * NET_MAX_STOICH), ('vmax', ct.c_double), ('keq', ct.c_double),
                ('term0', ct.c_int32), ('nterm', ct.c_int32)]


class BxNetSpec(ct.Structure):
    _fields_ = [('n_substances', ct.c_int32), ('n_reactions', ct.c_int32), ('n_terms', ct.c_int32),
                ('pad', ct.c_int32), ('substances', ct.POINTER(BxNetSubstance)),
                ('reactions', ct.POINTER(BxNetReaction)), ('terms', ct.POINTER(BxNetTerm)),
                ('mem_vol', _dp), ('R_rads', _dp)]


class BxState(ct.Structure):
    _fields_ = [('vm', _dp), ('cc_cells', _dp), ('cc_at_mem', _dp),
                ('cc_env', _dp), ('E_env_x', _dp), ('E_env_y', _dp), ('gjopen', _dp)]


OUTPUT_FIELDS = ['fluxes_mem', 'fluxes_gj', 'rate_NaKATP', 'rho_cells', 'Jn',
                 'I_mem', 'J_cell_x', 'J_cell_y', 'Jc', 'vm_ave', 'dvm',
                 'E_cell_x', 'E_cell_y', 'Emc', 'E_gj_x', 'E_gj_y', 'gjopen',
                 'sigma_cell', 'fluxes_env_x', 'fluxes_env_y', 'rho_env', 'v_env']


class BxOutputs(ct.Structure):
    _fields_ = [(n, _dp) for n in OUTPUT_FIELDS]


class BxStepStatus(ct.Structure):
    _fields_ = [('steps_done', ct.c_int64), ('nan_vm', ct.c_int32),
                ('nan_conc', ct.c_int32), ('neg_clamped', ct.c_int64),
                ('unstable', ct.c_int32), ('precision', ct.c_int32)]


class BxGraphLevel(ct.Structure):
    _fields_ = [('n', ct.c_int32), ('nnz', ct.c_int32), ('row_ptr', _ip), ('col', _ip), ('val', _dp)]


class BxGenSpec(ct.Structure):
    _fields_ = [('seed', ct.c_uint32), ('grid_size', ct.c_int32), ('nbx', ct.c_int32),
                ('nby', ct.c_int32), ('nrx', ct.c_int32), ('nry', ct.c_int32)] + \
        [(n, ct.c_double) for n in ('bx0', 'bx1', 'by0', 'by1', 'rx0', 'rx1', 'ry0', 'ry1', 'jitter',
                                    'radius', 'd_cell', 'cell_radius', 'scale_cell', 'cell_height')]


GEN_ARRAYS = [('cell_mem_ptr', 'i'), ('nn_i', 'i'), ('map_mem2ecm', 'i'), ('mem_sa', 'd'),
              ('mem_nx', 'd'), ('mem_ny', 'd'), ('R_rads', 'd'), ('mem_mid_x', 'd'),
              ('mem_mid_y', 'd'), ('cell_vol', 'd'), ('cell_sa', 'd'), ('diviterm', 'd'),
              ('cell_centre_x', 'd'), ('cell_centre_y', 'd'), ('mem_sa_per_env', 'd'),
              ('cell_nn_ptr', 'i'), ('cell_nn', 'i'), ('lattice_x', 'd'), ('lattice_y', 'd')]


class BxGenArrays(ct.Structure):
    _fields_ = [(n, _ip if t == 'i' else _dp) for n, t in GEN_ARRAYS]


# every symbol include/bx.h declares: name -> (restype, argtypes)
SIGNATURES = {
    'bx_cluster_create': (ct.c_int, [ct.POINTER(BxGeom), ct.POINTER(BxParams), ct.c_int,
                                     ct.POINTER(ct.c_void_p)]),
    'bx_batch_create': (ct.c_int, [ct.POINTER(BxGeom), ct.POINTER(BxParams), ct.c_int, ct.c_int,
                                   ct.POINTER(ct.c_void_p)]),
    'bx_batch_layout': (ct.c_int, [ct.c_void_p, _ip, _ip]),
    'bx_batch_set_params': (ct.c_int, [ct.c_void_p, ct.POINTER(BxParams)]),
    'bx_destroy': (None, [ct.c_void_p]),
    'bx_set_membrane_diffusivity': (ct.c_int, [ct.c_void_p, _dp]),
    'bx_set_env_diffusivity': (ct.c_int, [ct.c_void_p, _dp]),
    'bx_set_boundary_potential': (ct.c_int, [ct.c_void_p, _dp]),
    'bx_set_params': (ct.c_int, [ct.c_void_p, ct.POINTER(BxParams)]),
    'bx_state_upload': (ct.c_int, [ct.c_void_p, ct.POINTER(BxState)]),
    'bx_state_download': (ct.c_int, [ct.c_void_p, ct.POINTER(BxState)]),
    'bx_step': (ct.c_int, [ct.c_void_p, ct.c_int, ct.c_int, ct.c_void_p]),
    'bx_outputs_download': (ct.c_int, [ct.c_void_p, ct.POINTER(BxOutputs)]),
    'bx_status': (ct.c_int, [ct.c_void_p, ct.POINTER(BxStepStatus)]),
    'bx_set_lap_env_inv': (ct.c_int, [ct.c_void_p, _dp]),
    'bx_build_lap_env_inv': (ct.c_int, [ct.c_void_p]),
    'bx_lap_env_inv_build': (ct.c_int, [ct.c_int, ct.c_int, ct.c_double, ct.c_void_p, ct.c_int64, ct.c_void_p]),
    'bx_max_abs_dvm': (ct.c_int, [ct.c_void_p, _dp]),
    'bx_batch_set_lap_env_inv': (ct.c_int, [ct.c_void_p, ct.c_int, ct.c_int, ct.c_double, _dp]),
    'bx_batch_env_fields': (ct.c_int, [ct.c_void_p, _dp, _dp, _dp, _dp, _dp, _dp, _dp]),
    'bx_dense_op_create': (ct.c_int, [_dp, ct.c_int, ct.POINTER(ct.c_void_p)]),
    'bx_dense_op_set_forward': (ct.c_int, [ct.c_void_p, _ip, _ip, _dp]),
    'bx_dense_op_apply': (ct.c_int, [ct.c_void_p, ct.c_void_p, ct.c_void_p, ct.c_int, ct.c_void_p,
                                     ct.c_int, ct.c_void_p]),
    'bx_dense_op_status': (ct.c_int, [ct.c_void_p, ct.POINTER(ct.c_int)]),
    'bx_dense_op_time': (ct.c_int, [ct.c_void_p, ct.c_void_p, ct.c_void_p, ct.c_int, ct.c_int,
                                    ct.POINTER(ct.c_double)]),
    'bx_dense_op_destroy': (ct.c_int, [ct.c_void_p]),
    'bx_dense_op_create_empty': (ct.c_int, [ct.c_int, ct.POINTER(ct.c_void_p)]),
    'bx_dense_op_set_columns': (ct.c_int, [ct.c_void_p, ct.c_int, ct.c_int, ct.c_void_p, ct.c_void_p]),
    'bx_graph_create': (ct.c_int, [ct.c_int, ct.POINTER(BxGraphLevel), _dp, ct.POINTER(BxGraphLevel), _dp,
                                   ct.c_int, ct.POINTER(ct.c_void_p)]),
    'bx_graph_solve': (ct.c_int, [ct.c_void_p, ct.c_void_p, ct.c_void_p, ct.c_int, ct.c_double, ct.c_int,
                                  ct.POINTER(ct.c_int), ct.POINTER(ct.c_double), ct.c_void_p]),
    'bx_lap_gj_apply': (ct.c_int, [ct.c_void_p, ct.c_void_p, ct.c_void_p, ct.c_int, ct.c_double, ct.c_int,
                                   ct.POINTER(ct.c_int), ct.POINTER(ct.c_double), ct.c_void_p]),
    'bx_lap_gj_dense': (ct.c_int, [ct.c_void_p, ct.c_double, ct.c_int, ct.POINTER(ct.c_int),
                                   ct.POINTER(ct.c_double), ct.c_void_p, ct.POINTER(ct.c_void_p)]),
    'bx_graph_destroy': (ct.c_int, [ct.c_void_p]),
    'bx_gnn_create': (ct.c_int, [ct.POINTER(ct.c_void_p)]),
    'bx_gnn_n_params': (ct.c_int, []),
    'bx_gnn_set_params': (ct.c_int, [ct.c_void_p, _fp]),
    'bx_gnn_get_params': (ct.c_int, [ct.c_void_p, _fp]),
    'bx_gnn_set_graph': (ct.c_int, [ct.c_void_p, ct.c_int, _ip, _ip]),
    'bx_gnn_forward': (ct.c_int, [ct.c_void_p, ct.c_int, ct.c_int, ct.c_void_p, ct.c_int, ct.c_void_p,
                                  ct.c_int]),
    'bx_gnn_gradients': (ct.c_int, [ct.c_void_p, ct.c_int, ct.c_int, ct.c_void_p, ct.c_int, ct.c_void_p,
                                    ct.c_int, _fp, _fp]),
    'bx_gnn_train_step': (ct.c_int, [ct.c_void_p, ct.c_int, ct.c_int, ct.c_void_p, ct.c_int, ct.c_void_p,
                                     ct.c_int, ct.c_float, _fp]),
    'bx_gnn_destroy': (ct.c_int, [ct.c_void_p]),
    'bx_env_fields': (ct.c_int, [ct.c_void_p, _dp, _dp, _dp, _dp, _dp, _dp, _dp]),
    'bx_time_env_fields': (ct.c_int, [ct.c_void_p, ct.c_int, ct.POINTER(ct.c_double),
                                      ct.POINTER(ct.c_double)]),
    'bx_dense_apply_f64': (ct.c_int, [ct.c_void_p, ct.c_void_p, ct.c_void_p, ct.c_int,
                                      ct.c_int, ct.c_void_p]),
    'bx_abi_version': (ct.c_int, []),
    'bx_last_error': (ct.c_char_p, []),
    'bx_launch_count': (ct.c_int64, [ct.c_void_p]),
    'bx_cluster_info': (ct.c_int, [ct.c_void_p, _ip]),
    'bx_time_cell_kernel': (ct.c_int, [ct.c_void_p, ct.c_int, ct.POINTER(ct.c_double)]),
    'bx_cell_kernel_bytes': (ct.c_int64, [ct.c_void_p]),
    'bx_fp64_fma_probe': (ct.c_int, [ct.c_int, ct.c_int, ct.c_double, ct.c_double, ct.c_void_p, ct.c_void_p]),
    'bx_set_launch_config': (ct.c_int, [ct.c_void_p, ct.c_int, ct.c_int]),
    'bx_get_launch_config': (ct.c_int, [ct.c_void_p, ct.POINTER(ct.c_int), ct.POINTER(ct.c_int)]),
    'bx_autotune': (ct.c_int, [ct.c_void_p, ct.c_int, ct.POINTER(ct.c_int), ct.POINTER(ct.c_double)]),
    'bx_resident_info': (ct.c_int, [ct.c_void_p, ct.POINTER(ct.c_int), ct.POINTER(ct.c_int),
                                    ct.POINTER(ct.c_int), ct.POINTER(ct.c_int64)]),
    'bx_resident_barrier_check': (ct.c_int, [ct.c_void_p, ct.c_int64, ct.POINTER(ct.c_int)]),
    'bx_autotune_table': (ct.c_int, [ct.c_void_p, ct.c_int, ct.c_int, ct.POINTER(ct.c_int), _ip, _ip, _ip, _dp]),
    'bx_network_create': (ct.c_int, [ct.c_void_p, ct.POINTER(BxNetSpec), ct.POINTER(ct.c_void_p)]),
    'bx_network_upload': (ct.c_int, [ct.c_void_p, ct.c_void_p, ct.c_void_p, ct.c_void_p]),
    'bx_network_download': (ct.c_int, [ct.c_void_p, ct.c_void_p, ct.c_void_p, ct.c_void_p]),
    'bx_network_step': (ct.c_int, [ct.c_void_p, ct.c_int, ct.c_int, ct.c_int]),
    'bx_network_fluxes': (ct.c_int, [ct.c_void_p, ct.c_void_p, ct.c_void_p, ct.c_void_p]),
    'bx_network_status': (ct.c_int, [ct.c_void_p, ct.POINTER(ct.c_int64)]),
    'bx_network_destroy': (ct.c_int, [ct.c_void_p]),
    'bx_network_info': (ct.c_int, [ct.c_void_p, _ip]),
    'bx_network_time_step': (ct.c_int, [ct.c_void_p, ct.c_int, ct.c_int, ct.POINTER(ct.c_double)]),
    'bx_step_fp64_noalloc': (ct.c_int, [ct.POINTER(BxGeom), ct.POINTER(BxParams), ct.c_void_p,
                                        ct.c_void_p, ct.c_void_p, ct.c_void_p, ct.c_void_p,
                                        ct.c_void_p, ct.c_void_p, ct.c_int, ct.c_void_p]),
    'bx_generate_cluster': (ct.c_int, [ct.POINTER(BxGenSpec), ct.c_void_p, ct.POINTER(ct.c_void_p)]),
    'bx_generated_info': (ct.c_int, [ct.c_void_p, _ip, _dp]),
    'bx_generated_download': (ct.c_int, [ct.c_void_p, ct.POINTER(BxGenArrays)]),
    'bx_generated_destroy': (ct.c_int, [ct.c_void_p]),
}

_lib = None


def load(path: str = LIB_PATH):
    """Load libbx.so (once) and declare its signatures."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise BxLibraryError(
            f'{path} is missing: build it with betse_gb300.build.build() '
            '(there is no CPU fallback for the step)')
    try:
        lib = ct.CDLL(path)
    except OSError as e:
        raise BxLibraryError(f'cannot load {path}: {e}') from e
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(rc: int, what: str) -> None:
    if rc != BX_OK:
        msg = load().bx_last_error()
        msg = msg.decode() if msg else ''
        raise BxLibraryError(f'{what} failed ({rc}): {msg}')


def dptr(a):
    """double* of a C-contiguous float64 numpy array (or None)."""
    if a is None:
        return None
    return a.ctypes.data_as(_dp)


def iptr(a):
    return a.ctypes.data_as(_ip)


def u8ptr(a):
    return a.ctypes.data_as(_u8p)
