#!/usr/bin/env python3
"""Generate the golden fixtures under ``tests/golden/`` by running BETSE itself.

This script is test infrastructure. It imports the reference BETSE sources
(pure Python/NumPy) from a local checkout, builds a seeded cell cluster with
BETSE's own ``Cells`` code, runs BETSE's own ``Simulator`` time loop
(``betse/science/sim.py:1132-1390``) and stores, in small ``.npz`` files:

* the cluster geometry and index maps exactly as ``Cells`` built them,
* the initial state after ``init_core``/``init_dynamics``/``update_V``,
* the state and the step outputs after selected step counts.

The checkout cannot travel with the repository, so the fixtures are committed
and the tests read only them. Run it from the repository root::

    python tests/golden/make_golden.py --ref <path of a BETSE checkout>

BETSE's package ``__init__`` modules pull in beartype, dill, matplotlib,
ruamel.yaml and PIL, none of which the hot path uses. The loader below stubs
those imports and bypasses ``betse.science.__init__`` (which only initialises
the application's plotting stack); every module on the hot path is imported
unmodified from the checkout.

Workload recipe (mirrors ``Cells.make_world``, ``betse/science/cells.py:414``):
hexagonal seed lattice with disorder 0.4 (``cells.py:742-801``), the DEC mesh
clipped to a circle (``cells.py:930-944``, ``math/mesh.py:189``), then
``cell_index, cellVerts, cellMatrices, cell_vols, mem_processing, near_neigh,
makeECM, environment`` and ``makeLaplacian`` (``cells.py:503``).
"""
from __future__ import annotations

import argparse
import importlib.abc
import importlib.machinery
import os
import sys
import time
import types
import typing
from types import SimpleNamespace
from unittest.mock import MagicMock

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


# --------------------------------------------------------------------------
# Headless loader for the reference checkout
# --------------------------------------------------------------------------
def install_reference(ref: str) -> None:
    bt = types.ModuleType('beartype')
    bt.__path__ = []
    bt.beartype = lambda f=None, **kw: f if f is not None else (lambda g: g)

    class BeartypeConf:
        def __init__(self, *a, **k):
            pass
    bt.BeartypeConf = BeartypeConf
    claw = types.ModuleType('beartype.claw')
    claw.beartype_this_package = lambda *a, **k: None
    claw.beartype_package = lambda *a, **k: None
    btt = types.ModuleType('beartype.typing')
    for n in dir(typing):
        setattr(btt, n, getattr(typing, n))
    sys.modules.update({'beartype': bt, 'beartype.claw': claw,
                        'beartype.typing': btt})
    mocked = ('dill', 'matplotlib', 'ruamel', 'PIL', 'yaml', 'mpl_toolkits',
              'pydot', 'beartype.vale', 'beartype.door', 'beartype.roar')

    class Finder(importlib.abc.MetaPathFinder, importlib.abc.Loader):
        def find_spec(self, name, path, target=None):
            if any(name == m or name.startswith(m + '.') for m in mocked):
                return importlib.machinery.ModuleSpec(name, self,
                                                      is_package=True)
            return None

        def create_module(self, spec):
            m = MagicMock(name=spec.name)
            m.__path__ = []
            m.__spec__ = spec
            return m

        def exec_module(self, module):
            pass

    sys.meta_path.insert(0, Finder())
    sys.path.insert(0, ref)
    import betse  # noqa: F401  (its __init__ only calls the stubbed claw)
    sci = types.ModuleType('betse.science')
    sci.__path__ = [os.path.join(ref, 'betse', 'science')]
    sys.modules['betse.science'] = sci
    betse.science = sci


# --------------------------------------------------------------------------
# Parameters (duck-typed stand-in for betse.science.parameters.Parameters)
# --------------------------------------------------------------------------
ION_ORDER = ['Na', 'K', 'Cl', 'Ca', 'P', 'M']   # order of p.ions_dict (H off)


def make_params(radius, grid_size, is_ecm, dt, n_steps, cell_space=26e-9, sharpness=1.0, v_sensitive_gj=False,
                alpha_Ca=0.0, cell_polarizability=0.0):
    from betse.science.enum.enumconf import CellLatticeType, SolverType
    p = SimpleNamespace()
    # physical constants, parameters.py:1087-1122
    p.F, p.R, p.eo, p.kb, p.q = 96485, 8.314, 8.854e-12, 1.3806e-23, 1.602e-19
    p.mu, p.NAv, p.er, p.eedl = 1.275e-6, 6.022e23, 80.0, 40.0
    p.deltaGATP = -37000
    p.cATP, p.cADP, p.cPi = 1.5, 0.1, 0.1
    p.KmNK_Na, p.KmNK_K, p.KmNK_ATP = 12.0, 0.2, 0.5
    p.KmCa_Ca, p.KmCa_ATP = 1.0e-3, 0.5
    p.z_Na, p.z_K, p.z_Cl, p.z_Ca, p.z_H, p.z_P, p.z_M = 1, 1, -1, 2, 1, -1, -1
    p.tm, p.ac, p.scale_cell = 7.5e-9, 1.0e-6, 0.99
    # workload: 37 C, cm 0.022 F/m2, alpha_NaK 5e-8
    p.T = 310.15
    p.cm = 0.022
    p.alpha_NaK = 5e-8
    p.alpha_Ca = alpha_Ca   # Ca-ATPase rate (sim_config.yaml default 5e-8; 0 turns ca_handler's pump off)
    p.dt = dt
    p.cell_radius = 5e-6
    p.d_cell = 2 * p.cell_radius
    p.cell_lattice_type = CellLatticeType.HEX
    p.cell_lattice_disorder = 0.4
    p.cell_height = 1e-5
    p.cell_space = cell_space
    p.world_len = 2 * radius + 20e-6
    p.wsx = p.wsy = p.world_len
    p.nx = int(p.wsx / p.d_cell)
    p.ny = int(p.wsy / p.d_cell)
    p.wsx = p.wsx + 5 * p.cell_lattice_disorder * p.d_cell
    p.wsy = p.wsy + 5 * p.cell_lattice_disorder * p.d_cell
    p.vol_env = 1.0 * p.wsx * p.wsy * p.cell_height
    p.gjl = 2 * p.tm + p.cell_space
    p.grid_size = grid_size
    p.is_ecm = is_ecm
    p.cluster_open = True
    p.sharpness = sharpness
    p.smooth_cells = 1 / 0.5
    p.true_cell_size = 1.0e-5
    p.cell_polarizability = cell_polarizability
    p.gj_surface = 5.0e-8
    p.v_sensitive_gj = v_sensitive_gj
    # gating constants of sim_config.yaml's 'gap junctions' block
    p.gj_vthresh, p.gj_vgrad, p.gj_min = 15.0, 15.0, 0.10
    p.fast_update_ecm = False
    p.D_tj, p.D_adh = 1.0, 1.0
    p.channel_noise_level = 0.0
    p.dynamic_noise = 0
    p.dynamic_noise_level = 0.0
    p.molecules_enabled = False
    p.grn_enabled = False
    p.deform_osmo = False
    p.fluid_flow = False
    p.deformation = False
    p.td_deform = False
    p.Ca_dyn = 0
    p.cbnd = None
    p.svg_override = False
    p.single_cell = False
    p.alpha_shape = 0.4
    p.use_centroids = True
    p.refine_mesh = False
    p.maximum_voronoi_steps = 25
    p.voronoi_convergence = 7.5
    p.global_options = {'gj_block': 0, 'NaKATP_block': 0}
    p.solver_type = SolverType.FULL
    p.sim_ECM = is_ecm
    p.init_tsteps = n_steps
    p.sim_tsteps = n_steps
    p.run_sim = False
    # ions: Na/K/Cl/Ca/P in and out, M balancing charge (parameters.py:1569)
    p.ions_dict = {'Na': 1, 'K': 1, 'Cl': 1, 'Ca': 1, 'H': 0, 'P': 1, 'M': 1}
    # P inside is not fixed by the workload; 100 mM (the reference's amphibian
    # profile, parameters.py:1416, which shares Na 8 / K 125) keeps M an anion.
    cell = {'Na': 8.0, 'K': 125.0, 'Cl': 10.0, 'Ca': 1e-4, 'P': 100.0}
    env = {'Na': 145.0, 'K': 5.0, 'Cl': 105.0, 'Ca': 1.0, 'P': 10.0}
    zs = {'Na': 1, 'K': 1, 'Cl': -1, 'Ca': 2, 'P': -1}
    cell['M'] = abs(-sum(cell[k] * zs[k] for k in cell))
    env['M'] = abs(-sum(env[k] * zs[k] for k in env))
    p.cell_concs, p.env_concs = cell, env
    p.ion_charge = {'Na': 1, 'K': 1, 'Cl': -1, 'Ca': 2, 'P': -1, 'M': -1}
    p.free_diff = {'Na': 1.33e-9, 'K': 1.96e-9, 'Cl': 2.03e-9,
                   'Ca': 1.0e-10, 'P': 0.0, 'M': 1.0e-9}
    p.mem_perms = {'Na': 1e-18, 'K': 1e-18, 'Cl': 1e-18, 'Ca': 1e-18,
                   'P': 0.0, 'M': 1e-18}
    p.molar_mass = {'Na': 23e-3, 'K': 39e-3, 'Cl': 35e-3, 'Ca': 40e-3,
                    'P': 500e-3, 'M': 60e-3}
    p.ion_long_name = {k: k for k in p.ions_dict}
    p.Dtj_rel = {k: 1.0 for k in p.ions_dict}
    p.cCa_er = 0.5
    return p


class CircleMask:
    """Duck-typed image mask: a disc of radius ``r`` about ``centre``."""

    def __init__(self, centre, r, n_poly=256, msize=64):
        self.cx, self.cy, self.r = float(centre[0]), float(centre[1]), r
        th = np.linspace(0, 2 * np.pi, n_poly, endpoint=False)
        self.clipcurve = np.column_stack((self.cx + r * np.cos(th),
                                          self.cy + r * np.sin(th)))
        self.msize = msize
        self.clipping_matrix = np.ones((msize, msize))

    def clipping_function(self, x, y):
        return 1.0 if (x - self.cx) ** 2 + (y - self.cy) ** 2 <= self.r ** 2 else 0.0


def build_cells(p, radius, seed):
    from betse.science.cells import Cells
    from betse.science.math.mesh import DECMesh
    np.random.seed(seed)
    c = Cells.__new__(Cells)
    c.p = p
    c._make_cell_lattice(p)
    mask = CircleMask(c.centre, radius)
    c.mesh = DECMesh(cell_radius=p.cell_radius, seed_points=c.clust_xy,
                     alpha_shape=p.alpha_shape, use_centroids=p.use_centroids,
                     use_alpha_shape=True, single_cell_noise=0.5,
                     single_cell_sides=6, image_mask=None, allow_merging=True,
                     merge_thresh=0.1, close_thresh=0.1,
                     make_all_operators=False, mesh_type='tri')
    c.mesh.clip_and_refine(mask, smoothing=None, refinement=False,
                           max_steps=p.maximum_voronoi_steps,
                           convergence=p.voronoi_convergence, fix_bounds=True)
    c.ecm_verts = c.mesh.vcell_verts
    c.cluster_mask = mask.clipping_matrix
    c.msize = mask.msize
    c.ecm_verts_unique = c.mesh.vor_verts
    c.cell_index(p)
    c.cellVerts(p)
    c.cellMatrices(p)
    c.cell_vols(p)
    c.mem_processing(p)
    c.near_neigh(p)
    c.makeECM(p)
    c.environment(p)
    c.grid_len = len(c.xypts)
    bdic = {'N': 'value', 'S': 'value', 'E': 'value', 'W': 'value'}
    _, c.lapENVinv = c.grid_obj.makeLaplacian(bound=bdic)
    c.lapGJinv = None
    c.lapGJ = None
    c.cell_i = np.asarray(c.cell_i)
    c.gj_default_weights = np.ones(len(c.mem_i))
    return c


def draw_cluster_parameters(c, seed, dm_lo=1e-19, dm_hi=1e-17):
    """Per-membrane Dm (log-uniform, Dm_P = 0) and per-pair GJ weights."""
    rng = np.random.default_rng(seed + 1)
    n_m = len(c.mem_i)
    dm = np.exp(rng.uniform(np.log(dm_lo), np.log(dm_hi), size=(6, n_m)))
    dm[ION_ORDER.index('P')] = 0.0
    w = rng.uniform(0.5, 1.0, size=n_m)
    nn = np.asarray(c.nn_i)
    lo = np.minimum(np.arange(n_m), nn)
    w = w[lo]                     # the same value on m and nn_i[m]
    return dm, w


class _Fake:
    def __init__(self, dm):
        self.dm = dm

    def init_profiles(self, phase):
        phase.sim.Dm_cells = self.dm.copy()

    def init_events(self, phase):
        pass

    def fire_events(self, phase, t):
        pass

    def progressed_next(self, *a, **k):
        pass


STATE_KEYS = ['vm', 'cc_cells', 'cc_env', 'cc_at_mem']
OUT_KEYS = ['fluxes_mem', 'fluxes_gj', 'rate_NaKATP', 'rho_cells', 'Jn',
            'I_mem', 'J_cell_x', 'J_cell_y', 'Jc', 'vm_ave', 'dvm',
            'E_cell_x', 'E_cell_y', 'Emc', 'E_gj_x', 'E_gj_y', 'gjopen',
            'sigma_cell', 'Phi_b', 'v_env', 'E_env_x', 'E_env_y',
            'J_env_x', 'J_env_y', 'B_field']


def run_case(name, radius, seed, is_ecm, grid_size, dt, checkpoints,
             dm_range=(1e-19, 1e-17), cell_space=26e-9, sharpness=1.0, v_sensitive_gj=False,
             alpha_Ca=0.0, cell_polarizability=0.0, network=None):
    from betse.science.sim import Simulator
    from betse.science.enum.enumphase import SimPhaseKind
    n_steps = max(checkpoints)
    p = make_params(radius, grid_size, is_ecm, dt, n_steps, cell_space, sharpness, v_sensitive_gj, alpha_Ca,
                    cell_polarizability)
    t0 = time.time()
    c = build_cells(p, radius, seed)
    t_seed = time.time() - t0
    dm, w = draw_cluster_parameters(c, seed, *dm_range)
    c.gj_default_weights = w.copy()
    fake = _Fake(dm)
    phase = SimpleNamespace(p=p, cells=c, kind=SimPhaseKind.INIT, dyna=fake,
                            callbacks=fake)
    s = Simulator()
    phase.sim = s
    s.init_core(phase)
    s.init_dynamics(phase)
    s.clear_storage(c, p)
    s.update_V(c, p)
    out = {}
    core = attach_network(phase, network, out) if network else None
    # ---- geometry and index maps, exactly as Cells built them
    g = dict(
        mem_to_cells=np.asarray(c.mem_to_cells, np.int64),
        nn_i=np.asarray(c.nn_i, np.int64),
        bflags_mems=np.asarray(c.bflags_mems, np.int64),
        num_mems=np.asarray(c.num_mems, np.int64),
        mem_sa=c.mem_sa, cell_vol=c.cell_vol, cell_sa=c.cell_sa,
        diviterm=c.diviterm, mem_vects_flat=c.mem_vects_flat,
        R_rads=c.R_rads, map_mem2ecm=np.asarray(c.map_mem2ecm, np.int64),
        grid_shape=np.asarray(c.X.shape, np.int64), delta=np.float64(c.delta),
        gj_len=np.float64(c.gj_len), gj_default_weights=w,
        memSa_per_envSquare=c.memSa_per_envSquare,
        cell_centres=c.cell_centres, mem_mids_flat=c.mem_mids_flat,
        xypts=c.xypts, cell_nn_flat=np.concatenate(
            [np.asarray(v, np.int64) for v in c.cell_nn]) if len(c.cell_nn) else np.zeros(0, np.int64),
        cell_nn_ptr=np.cumsum([0] + [len(v) for v in c.cell_nn]).astype(np.int64),
    )
    if is_ecm:
        g.update(D_env=s.D_env, D_env_weight=s.D_env_weight, ko_env=np.float64(s.ko_env),
                 c_env_bound=np.asarray(s.c_env_bound, np.float64),
                 env_bound_idx=np.asarray(np.unique(np.concatenate(
                     [c.bBot_k, c.bTop_k, c.bL_k, c.bR_k])), np.int64))
    else:
        g.update(D_env_weight=s.D_env_weight)
    for k, v in g.items():
        out['geom_' + k] = np.asarray(v)
    sc = dict(F=p.F, R=p.R, T=s.T, dt=p.dt, cm=p.cm, tm=p.tm,
              gj_surface=p.gj_surface, alpha_NaK=p.alpha_NaK,
              KmNK_Na=p.KmNK_Na, KmNK_K=p.KmNK_K, KmNK_ATP=p.KmNK_ATP,
              cATP=p.cATP, cADP=p.cADP, cPi=p.cPi, deltaGATP=p.deltaGATP,
              vol_env=p.vol_env, cell_height=p.cell_height, q=p.q, kb=p.kb,
              eo=p.eo, er=p.er, mu=p.mu, sharpness=p.sharpness,
              cell_radius=p.cell_radius, true_cell_size=p.true_cell_size,
              sigma=np.float64(s.sigma), is_ecm=float(is_ecm),
              v_sensitive_gj=float(bool(v_sensitive_gj)), gj_vthresh=p.gj_vthresh, gj_min=p.gj_min,
              alpha_Ca=p.alpha_Ca, KmCa_Ca=p.KmCa_Ca, KmCa_ATP=p.KmCa_ATP,
              cell_polarizability=p.cell_polarizability)
    for k, v in sc.items():
        out['par_' + k] = np.float64(v)
    out['par_zs'] = np.asarray(s.zs, np.float64)
    out['par_D_free'] = np.asarray(s.D_free, np.float64)
    out['par_D_gj'] = np.asarray(s.D_gj, np.float64)[:, 0]
    out['par_smooth_weight_mem'] = s.smooth_weight_mem
    out['par_smooth_weight_o'] = s.smooth_weight_o
    out['par_Dm_cells'] = np.asarray(s.Dm_cells, np.float64)
    out['par_ion_names'] = np.asarray(ION_ORDER)
    state_keys = STATE_KEYS + (['gjopen'] if v_sensitive_gj else [])
    for k in state_keys:
        v = np.array(getattr(s, k), np.float64)
        out['init_' + k] = v * np.ones(len(c.mem_i)) if k == 'gjopen' else v
    cps = sorted(set(checkpoints))
    time_steps = np.arange(n_steps) * p.dt
    done = 0
    t_loop = 0.0
    for cp in cps:
        t0 = time.time()
        s._run_sim_core_loop(phase, time_steps[done:cp], set(), None)
        t_loop += time.time() - t0
        done = cp
        for k in state_keys:
            out[f's{cp}_' + k] = np.array(getattr(s, k), np.float64)
        if core is not None:
            save_network_state(core, out, f's{cp}_')
        for k in OUT_KEYS:
            if cp in cps[:2] and hasattr(s, k):
                v = getattr(s, k)
                out[f's{cp}_' + k] = np.array(v, np.float64)
    out['meta_seed'] = np.int64(seed)
    out['meta_radius'] = np.float64(radius)
    out['meta_checkpoints'] = np.asarray(cps, np.int64)
    out['meta_ms_per_step'] = np.float64(1e3 * t_loop / n_steps)
    path = os.path.join(HERE, name + '.npz')
    np.savez_compressed(path, **out)
    print(f'{name}: {len(c.cell_i)} cells, {len(c.mem_i)} mems, grid '
          f'{tuple(c.X.shape)}, seed {t_seed:.1f} s, '
          f'{1e3 * t_loop / n_steps:.2f} ms/step, '
          f'{os.path.getsize(path) / 1024:.0f} KiB')
    return out


# --------------------------------------------------------------------------
# Molecule networks (MasterOfNetworks, chemistry/networks.py)
# --------------------------------------------------------------------------
# A four-substance, two-reaction network written for these fixtures in the
# configuration format BETSE reads ('general network' -> 'biomolecules' and
# 'reactions'). Between them the entries use each influencer kind that
# get_influencers composes (networks.py:5084-5600): multiplicative, '!'
# independent and '&' direct activators, inhibitors, an 'env'-zone inhibitor
# and decay activators; growth restricted to a tissue profile and modulated by
# gradient_x; time dilation; 'update intracellular' on and off; a charged and
# neutral substances crossing the membrane and the gap junctions; one
# irreversible reaction and one with a standard free energy. Absent entries
# are the string 'None', as BETSE's YAML loader gives them.
def _plot_block():
    return {'plot 2D': False, 'animate': False, 'autoscale colorbar': True, 'max val': 1.0, 'min val': 0.0}


def _substance(name, z, Dm, Do, Dgj, env, cell, gad, update_intra=False, gj_impermeable=False,
               time_dilation=False):
    return {'name': name, 'Dm': Dm, 'Do': Do, 'Dgj': Dgj, 'z': z, 'env conc': env, 'cell conc': cell,
            'update intracellular': update_intra, 'use time dilation': time_dilation,
            'TJ permeable': False, 'GJ impermeable': gj_impermeable, 'TJ factor': 1.0,
            'growth and decay': gad, 'plotting': _plot_block()}


NETWORK_SUBSTANCES = [
    _substance('A', 0, 0.0, 1.0e-12, 2.0e-15, 0.0, 0.1,
               {'production rate': 0.5, 'decay rate': 0.2, 'apply to': 'all',
                'modulator function': 'gradient_x', 'activators': 'None', 'Km activators': 'None',
                'n activators': 'None', 'inhibitors': ['C'], 'Km inhibitors': [0.3], 'n inhibitors': [2.0]}),
    _substance('B', 0, 0.0, 1.0e-12, 1.0e-15, 0.0, 0.05,
               {'production rate': 1.0, 'decay rate': 0.5, 'apply to': ['spot'],
                'modulator function': 'None', 'activators': ['A', 'C!'], 'Km activators': [0.2, 0.5],
                'n activators': [2.0, 1.0], 'inhibitors': 'None', 'Km inhibitors': 'None', 'n inhibitors': 'None',
                'decay max': 0.3, 'decay activators': ['A'], 'Km decay activators': [0.4],
                'n decay activators': [1.0]}, gj_impermeable=True),
    _substance('C', -1, 1.0e-18, 1.0e-11, 1.0e-14, 0.5, 0.2,
               {'production rate': 0.2, 'decay rate': 0.1, 'apply to': 'all', 'modulator function': 'None',
                'activators': ['B', 'A&'], 'Km activators': [0.1, 1.0], 'n activators': [1.0, 1.0],
                'inhibitors': 'None', 'Km inhibitors': 'None', 'n inhibitors': 'None'}),
    _substance('D', 0, 5.0e-19, 1.0e-11, 1.0e-15, 1.0, 0.1,
               {'production rate': 0.05, 'decay rate': 0.05, 'apply to': 'all', 'modulator function': 'None',
                'activators': 'None', 'Km activators': 'None', 'n activators': 'None',
                'inhibitors': ['C'], 'zone inhibitors': ['env'], 'Km inhibitors': [0.4],
                'n inhibitors': [1.0]}, update_intra=True, time_dilation=True),
]

NETWORK_REACTIONS = [
    {'name': 'r1', 'reaction zone': 'cell', 'reactants': ['A', 'C'], 'reactant multipliers': [1, 1],
     'Km reactants': [0.1, 0.2], 'products': ['D'], 'product multipliers': [1], 'Km products': [0.5],
     'max rate': 0.01, 'standard free energy': 'None', 'reaction activators': ['B'], 'activator Km': [0.1],
     'activator n': [2.0]},
    {'name': 'r2', 'reaction zone': 'cell', 'reactants': ['D'], 'reactant multipliers': [1],
     'Km reactants': [0.3], 'products': ['B'], 'product multipliers': [2], 'Km products': [0.4],
     'max rate': 0.02, 'standard free energy': -5000.0, 'reaction inhibitors': ['A'], 'inhibitor Km': [0.5],
     'inhibitor n': [1.0]},
]

NETWORK = dict(substances=NETWORK_SUBSTANCES, reactions=NETWORK_REACTIONS, time_dilation=2.0,
               spot_fraction=0.3, gradient_x={'x-offset': 0.1, 'exponent': 3.0, 'slope': 1.0, 'z-offset': 0.2})


def attach_network(phase, net, out):
    """Build BETSE's MasterOfNetworks the way MasterOfMolecules.read_mol_config
    does (chemistry/molecules.py) and hook it into the step loop
    (sim.py:1290-1303, p.molecules_enabled)."""
    from betse.science.chemistry.networks import MasterOfNetworks
    sim, cells, p = phase.sim, phase.cells, phase.p
    p.substances_affect_charge = False
    p.gradient_x_properties = dict(net['gradient_x'])
    rng = np.random.default_rng(1234)
    n_c = len(cells.cell_i)
    spot = np.sort(rng.choice(n_c, size=max(1, int(net['spot_fraction'] * n_c)), replace=False))
    phase.dyna.cell_target_inds = {'spot': list(spot)}
    mem_spot = np.nonzero(np.isin(np.asarray(cells.mem_to_cells), spot))[0]
    phase.dyna.tissue_target_inds = {'spot': list(mem_spot)}
    core = MasterOfNetworks(sim, cells, net['substances'], p)
    core.time_dila = float(net['time_dilation'])
    core.read_substances(sim, cells, net['substances'], p)
    core.tissue_init(phase, net['substances'])
    core.read_reactions(net['reactions'], sim, cells, p)
    core.write_reactions()
    core.create_reaction_matrix()
    core.write_reactions_env()
    core.create_reaction_matrix_env()
    sim.molecules = SimpleNamespace(core=core, transporters=False, channels=False, modulators=False)
    p.molecules_enabled = True
    import json
    out['net_config'] = np.asarray(json.dumps({'substances': net['substances'], 'reactions': net['reactions'],
                                               'time_dilation': net['time_dilation']}))
    out['net_spot_cells'] = spot.astype(np.int64)
    out['net_names'] = np.asarray(list(core.molecules))
    out['net_reaction_matrix'] = np.asarray(core.reaction_matrix)
    out['net_mem_vol'] = np.asarray(cells.mem_vol, np.float64)
    out['net_growth_mod'] = np.stack([np.asarray(m.growth_mod_function_cells, np.float64) *
                                      np.ones(n_c) if m.simple_growth else np.ones(n_c)
                                      for m in core.molecules.values()])
    save_network_state(core, out, 'init_')
    return core


def save_network_state(core, out, prefix):
    mols = list(core.molecules.values())
    out[prefix + 'net_c_cells'] = np.stack([np.array(m.c_cells, np.float64) for m in mols])
    out[prefix + 'net_cc_at_mem'] = np.stack([np.array(m.cc_at_mem, np.float64) for m in mols])
    out[prefix + 'net_c_env'] = np.stack([np.array(m.c_env, np.float64) for m in mols])
    if prefix != 'init_':
        out[prefix + 'net_f_mem'] = np.stack([np.array(m.f_mem, np.float64) * np.ones(len(m.cc_at_mem))
                                              for m in mols])
        out[prefix + 'net_f_gj'] = np.stack([np.array(m.f_gj, np.float64) * np.ones(len(m.cc_at_mem))
                                             for m in mols])



CASES = {
    # the 250-cell plain FP64 workload, no ECM, dt 1e-2, 2000 steps
    'noecm_r80_s1': dict(radius=80e-6, seed=1, is_ecm=False, grid_size=20,
                         dt=1e-2, checkpoints=[1, 2, 10, 100, 2000]),
    # a second seed and size, short run
    'noecm_r50_s7': dict(radius=50e-6, seed=7, is_ecm=False, grid_size=20,
                         dt=1e-2, checkpoints=[1, 25]),
    # extracellular spaces on (finite-volume environment grid), 25 nm cleft
    'ecm_r50_s3': dict(radius=50e-6, seed=3, is_ecm=True, grid_size=20,
                       dt=5e-3, checkpoints=[1, 2, 50], cell_space=25e-9),
    # extracellular spaces with environment smoothing (fd.integrator, sharpness < 1)
    'ecm_r40_s5_sharp': dict(radius=40e-6, seed=5, is_ecm=True, grid_size=20,
                             dt=5e-3, checkpoints=[1, 2, 30], cell_space=25e-9, sharpness=0.5),
    # voltage-gated gap junctions (BETSE's default 'voltage sensitive gj: True')
    'noecm_r50_s9_vgj': dict(radius=50e-6, seed=9, is_ecm=False, grid_size=20,
                             dt=1e-2, checkpoints=[1, 2, 40], v_sensitive_gj=True),
    # Ca-ATPase on (ca_handler; the mammal profile with sim_config.yaml's alpha_Ca)
    # together with voltage-gated gap junctions
    'noecm_r50_s11_ca': dict(radius=50e-6, seed=11, is_ecm=False, grid_size=20,
                             dt=1e-2, checkpoints=[1, 2, 40], alpha_Ca=5e-8, v_sensitive_gj=True),
    # Ca-ATPase with extracellular spaces and environment smoothing: the pump
    # reads the environment after that step's Nernst-Planck update
    'ecm_r40_s13_ca': dict(radius=40e-6, seed=13, is_ecm=True, grid_size=20,
                           dt=5e-3, checkpoints=[1, 2, 30], cell_space=25e-9, sharpness=0.5,
                           alpha_Ca=5e-8),
    # cell polarizability on: the implicit membrane-voltage update of update_V
    # (the value phasereqs.py sets when a phase asks for it)
    'noecm_r50_s17_pol': dict(radius=50e-6, seed=17, is_ecm=False, grid_size=20,
                              dt=1e-2, checkpoints=[1, 2, 40], cell_polarizability=1e-4),
    # a molecule network (MasterOfNetworks.run_loop) stepped with the ions
    'net_r50_s21': dict(radius=50e-6, seed=21, is_ecm=False, grid_size=20,
                        dt=1e-2, checkpoints=[1, 2, 50, 300], network=NETWORK),
    # a handful of cells: boundary-dominated edge case
    'noecm_r20_s2': dict(radius=20e-6, seed=2, is_ecm=False, grid_size=12,
                         dt=1e-2, checkpoints=[1, 20]),
}


def graph_case(name, radius, seed):
    """BETSE's Cells.graphLaplacian (cells.py:1845-1894) on a seeded cluster:
    the DEC-mesh inputs it reads (triangulation edges with their incidence
    signs, edge lengths, Voronoi areas), the lapGJinv and lapGJ it builds, and
    the product pressures.osmotic_P forms with it (physics/pressures.py:59,
    sim.PP = lapGJinv @ (-div_u_osmo * rho * dt)) on a seeded divergence."""
    p = make_params(radius, 20, False, 1e-2, 1)
    c = build_cells(p, radius, seed)
    c.graphLaplacian(p)
    m = c.mesh
    D = np.asarray(m.delta_tri_0)
    e = np.asarray(m.tri_edges, np.int64)
    rows = np.arange(len(e))
    assert np.all(D[rows, e[:, 0]] == -1) and np.all(D[rows, e[:, 1]] == 1)
    assert np.all((D != 0).sum(axis=1) == 2)
    rng = np.random.default_rng(seed + 100)
    div_u = rng.standard_normal(D.shape[1]) * 1e-3
    rho, dt = 1000.0, p.dt
    out = dict(mesh_tri_edges=e, mesh_tri_edge_len=np.asarray(m.tri_edge_len),
               mesh_vor_edge_len=np.asarray(m.vor_edge_len), mesh_vor_sa=np.asarray(m.vor_sa),
               lapGJinv=np.asarray(c.lapGJinv), lapGJ=np.asarray(c.lapGJ),
               press_div_u_osmo=div_u, press_rho=np.float64(rho), press_dt=np.float64(dt),
               press_PP=np.dot(c.lapGJinv, -div_u * rho * dt))
    path = os.path.join(HERE, name + '.npz')
    np.savez_compressed(path, **out)
    print(f'{name}: {D.shape[1]} cells, {len(e)} edges -> {path}')


GRAPH_CASES = {'lapgj_r80_s1': dict(radius=80e-6, seed=1)}


def lattice_cases(name, cases):
    """BETSE's seed lattice (Cells._make_cell_lattice, cells.py:742-801) and the
    cells it clips from it (DECMesh.clip_and_refine, cellVerts, cell_vols,
    mem_processing, near_neigh) for each (radius, seed): what the synthetic
    cluster generator is checked against."""
    out = {}
    for key, (radius, seed) in cases.items():
        p = make_params(radius, 20, False, 1e-2, 1)
        c = build_cells(p, radius, seed)
        out.update({f'{key}_xypts': np.asarray(c.clust_xy)[:-4], f'{key}_wsx': np.float64(p.wsx),
                    f'{key}_centre': np.asarray(c.centre), f'{key}_cell_centres': np.asarray(c.cell_centres),
                    f'{key}_mem_to_cells': np.asarray(c.mem_to_cells, np.int64),
                    f'{key}_nn_i': np.asarray(c.nn_i, np.int64),
                    f'{key}_bflags_mems': np.asarray(c.bflags_mems, np.int64),
                    f'{key}_mem_sa': np.asarray(c.mem_sa), f'{key}_cell_vol': np.asarray(c.cell_vol)})
        print(f'{name}/{key}: {len(c.cell_centres)} cells, {len(c.mem_i)} membranes')
    path = os.path.join(HERE, name + '.npz')
    np.savez_compressed(path, **out)
    print(f'-> {path}')


LATTICE_CASES = {'cells_lattice': {'r80_s1': (80e-6, 1), 'r50_s7': (50e-6, 7), 'r50_s3': (50e-6, 3)}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument('--ref', default=os.environ.get('BETSE_REF'),
                    help='path of a BETSE source checkout (or set BETSE_REF)')
    ap.add_argument('--only', default=None)
    a = ap.parse_args()
    if not a.ref:
        ap.error('give --ref <path of a BETSE checkout> or set BETSE_REF')
    install_reference(a.ref)
    for name, kw in CASES.items():
        if a.only and name not in a.only.split(','):
            continue
        run_case(name, **kw)
    for name, kw in GRAPH_CASES.items():
        if a.only and name not in a.only.split(','):
            continue
        graph_case(name, **kw)
    for name, cases in LATTICE_CASES.items():
        if a.only and name not in a.only.split(','):
            continue
        lattice_cases(name, cases)


if __name__ == '__main__':
    main()
