#!/usr/bin/env python
"""Benchmark: D3Q19 Shan-Chen time step, MLUPS and fraction of the HBM roofline.

Workload (one "step" = one lattice time step over the whole box): D3Q19, E6
isotropic force stencil, MRT collision with every relaxation rate 1.0, Guo
forcing, psi = exp(-1/rho), G = -5.0, 256^3 periodic box, a spherical droplet
of radius 40 (tanh width 2, rho_l = 2.2, rho_g = 0.15, 1e-4 seeded noise),
populations stored as FP32 deviations from w_q*rho0.  The FP64 path on the
same workload is reported beside it.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

``--impl reference`` times the reference's own CPU implementation of the
step (its generated CTypes kernels, built from oracle/_ref) on the host cores,
one independent sample box per thread.  Multi-GPU: replicas only (every rank
runs its own box; no data exchange), launched one rank per GPU by torchrun.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
for _p in (ROOT, os.path.join(ROOT, 'idea.deploy_gb300')):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import numpy as np  # noqa: E402

METRIC = 'D3Q19 Shan-Chen MLUPS (E6 stencil, MRT, FP32-shifted populations)'
BOX = (256, 256, 256)
R, RHO_L, RHO_G, WIDTH, SEED, G = 40.0, 2.2, 0.15, 2.0, 1234, -5.0
Q = 19
WORKLOAD = ('D3Q19 E6 MRT (all rates 1.0) + Guo, psi=exp(-1/rho), G=-5.0, 256^3 periodic, '
            'droplet R=40 tanh width 2, rho_l=2.2 rho_g=0.15, 1e-4 seeded noise')
# the stable twin of the headline (G=-5 diverges in the reference as well):
# G=-4.5 with the 3D E6 flat-interface densities
G_STABLE, RHO_L_STABLE, RHO_G_STABLE = -4.5, 4.636, 0.147


def dist_env():
    ws = int(os.environ.get('WORLD_SIZE', '1'))
    rank = int(os.environ.get('RANK', '0'))
    local = int(os.environ.get('LOCAL_RANK', '0'))
    return ws, rank, local


class Dist:
    """Barrier and max-over-ranks (torch.distributed only when WORLD_SIZE > 1)."""

    def __init__(self):
        self.ws, self.rank, self.local = dist_env()
        self.pg = None
        if self.ws > 1:
            import torch
            import torch.distributed as tdist
            torch.cuda.set_device(self.local)
            tdist.init_process_group('nccl')
            self.torch, self.tdist = torch, tdist

    def barrier(self):
        if self.ws > 1:
            self.tdist.barrier()

    def max(self, x):
        if self.ws == 1:
            return x
        t = self.torch.tensor([float(x)], device='cuda')
        self.tdist.all_reduce(t, op=self.tdist.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.ws > 1:
            self.tdist.destroy_process_group()


# ----------------------------------------------------------------------------
# clocks sampled during the timed region
# ----------------------------------------------------------------------------
class Clocks:
    Q = ('index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,'
         'clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,'
         'clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap')

    def __init__(self, gpu):
        self.gpu, self.p, self.lines = gpu, None, []

    def start(self):
        try:
            self.p = subprocess.Popen(['nvidia-smi', '-i', str(self.gpu), '--query-gpu=' + self.Q,
                                       '--format=csv,noheader,nounits', '-lms', '100'],
                                      stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.p = None

    def stop(self):
        if self.p is None:
            return None
        self.p.terminate()
        try:
            out, _ = self.p.communicate(timeout=5)
        except subprocess.TimeoutExpired:
            self.p.kill()
            out, _ = self.p.communicate()
        rows = []
        for line in out.strip().splitlines():
            f = [x.strip() for x in line.split(',')]
            if len(f) >= 9:
                rows.append(f)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace('.', '').isdigit()]
        reasons = set()
        for r in rows:
            for name, v in zip(['hw_slowdown', 'hw_thermal_slowdown', 'sw_thermal_slowdown', 'sw_power_cap'],
                               r[5:9]):
                if v.strip().lower() in ('active', '1', 'yes'):
                    reasons.add(name)
        return {'sm_mhz': float(np.median(sm)) if sm else None,
                'sm_max_mhz': float(rows[0][2]) if rows[0][2].replace('.', '').isdigit() else None,
                'power_w_max': max(float(r[3]) for r in rows if r[3].replace('.', '').isdigit()),
                'samples': len(rows), 'reasons': sorted(reasons)}


# ----------------------------------------------------------------------------
# CPU: the reference's generated kernels (oracle/_ref) or the oracle port
# ----------------------------------------------------------------------------
def _ref_kernels(tag):
    import ctypes
    from oracle import make_ref
    if not os.path.exists(make_ref.MANIFEST):
        return None
    man = json.load(open(make_ref.MANIFEST))
    if tag not in man:
        return None
    make_ref.build()
    ent = man[tag]
    libs = {}
    for role, f in ent['files'].items():
        so = os.path.join(make_ref.REF_DIR, f['file'][:-2] + '.so')
        if not os.path.exists(so):
            return None
        fn = getattr(ctypes.CDLL(so), f['kernel'])
        fn.restype = ctypes.c_int
        libs[role] = fn
    return ent, libs


def cpu_reference(steps_total, threads, tag='d3q19_e6_mrt1_64', box=None):
    """Reference CTypes kernels, `threads` independent boxes, `steps_total` steps
    each; returns (MLUPS aggregated, seconds, cells per box, kind)."""
    import ctypes
    from sclbm.profiles import droplet
    got = _ref_kernels(tag)
    if got is None:
        return None
    ent, k = got
    box = tuple(ent['box'])
    V = int(np.prod(box))
    D = len(box)
    st = []
    for t in range(threads):
        n = np.ascontiguousarray(droplet(box, box[0] * 10 / 64, RHO_L, RHO_G, WIDTH, SEED + t).ravel())
        u = np.zeros(V * D)
        pop = np.zeros(V * Q)
        k['init'](ctypes.c_void_p(pop.ctypes.data), ctypes.c_void_p(n.ctypes.data), ctypes.c_void_p(u.ctypes.data))
        st.append([n, np.zeros(V), pop, np.zeros(V * Q)])

    def worker(s, nsteps):
        for _ in range(nsteps):
            n, psi, pop, pop2 = s
            k['density'](ctypes.c_void_p(n.ctypes.data), ctypes.c_void_p(psi.ctypes.data),
                         ctypes.c_void_p(pop.ctypes.data))
            k['step'](ctypes.c_void_p(pop2.ctypes.data), ctypes.c_void_p(pop.ctypes.data),
                      ctypes.c_void_p(n.ctypes.data), ctypes.c_void_p(psi.ctypes.data))
            s[2], s[3] = pop2, pop

    ths = [threading.Thread(target=worker, args=(s, steps_total)) for s in st]
    t0 = time.perf_counter()
    for th in ths:
        th.start()
    for th in ths:
        th.join()
    dt = time.perf_counter() - t0
    return threads * V * steps_total / dt / 1e6, dt, V, 'reference'


def cpu_port(steps_total, threads, box=(32, 32, 32)):
    """The oracle port (one box per thread) when the reference kernels are absent."""
    from oracle import oracle as O
    from sclbm import XIStencils, FStencils
    from sclbm.profiles import droplet
    x, f = XIStencils['D3Q19'], FStencils['D3E6']
    sims = []
    for t in range(threads):
        s = O.OracleSim(box, x['XIs'], x['Ws'], x['c2'], f['Es'], f['Ws'], G, rates=[1.0] * Q)
        s.set_fields(droplet(box, box[0] * 10 / 64, RHO_L, RHO_G, WIDTH, SEED + t))
        s.init_populations()
        sims.append(s)
    ths = [threading.Thread(target=s.run, args=(steps_total,)) for s in sims]
    t0 = time.perf_counter()
    for th in ths:
        th.start()
    for th in ths:
        th.join()
    dt = time.perf_counter() - t0
    V = int(np.prod(box))
    return threads * V * steps_total / dt / 1e6, dt, V, 'port'


def cpu_measure(target_s=15.0, threads=None):
    """Bounded CPU sample: calibrate one step, then run for about target_s."""
    threads = threads or os.cpu_count() or 1
    res = cpu_reference(1, threads)
    runner = cpu_reference
    if res is None:
        runner = cpu_port
        res = cpu_port(1, threads)
    mlups, dt, V, kind = res
    steps = max(1, int(target_s / max(dt, 1e-3)))
    mlups, dt, V, kind = runner(steps, threads)
    sample = '%d threads x %d steps of an independent %d-cell box (%s), %.1f s' % (
        threads, steps, V, 'the reference\'s generated CTypes kernels' if kind == 'reference' else 'oracle port',
        dt)
    return {'value': round(mlups, 3), 'unit': 'MLUPS', 'cores': threads, 'kind': kind, 'sample': sample}


# ----------------------------------------------------------------------------
# GPU arm
# ----------------------------------------------------------------------------
def peaks():
    try:
        return json.load(open(os.path.join(ROOT, 'MEASURED_PEAKS.json')))
    except Exception:
        return None


def make_sim(precision, device, literals='exact', box=None, g=None, rho0=None):
    from sclbm import _lib, XIStencils, FStencils
    x, f = XIStencils['D3Q19'], FStencils['D3E6']
    S = np.eye(Q)
    return _lib.Sim(3, box or BOX, x['XIs'], x['Ws'], x['c2'], f['Es'], f['Ws'], G if g is None else g,
                    collision=_lib.COLL_MRT, mrt_s=S,
                    precision=_lib.FP32_SHIFTED if precision == 'fp32' else _lib.FP64,
                    rho0=0.5 * (RHO_L + RHO_G) if rho0 is None else rho0, device=device,
                    literals={'exact': _lib.LIT_EXACT, 'factored': _lib.LIT_FACTORED}.get(literals, _lib.LIT_ROUND15))


def stable_twin(dev, steps, ms_headline):
    """The headline's kernel on the same box at the stable coupling G=-4.5:
    the step does the same work whatever the data (no branch depends on it),
    so its time should equal the headline's, which diverges to NaN."""
    from sclbm.profiles import droplet
    n0 = droplet(BOX, R, RHO_L_STABLE, RHO_G_STABLE, WIDTH, SEED)
    s = make_sim('fp32', dev, g=G_STABLE, rho0=0.5 * (RHO_L_STABLE + RHO_G_STABLE))
    s.set_density(n0)
    s.set_velocity(np.zeros(3 * n0.size))
    s.init_populations()
    s.step(5)
    ms = s.step_timed(steps)
    finite, nmax = s.density_finite()
    s.close()
    return {'G': G_STABLE, 'rho_l': RHO_L_STABLE, 'rho_g': RHO_G_STABLE, 'steps': steps,
            'ms_per_step': round(ms / steps, 5), 'value': round(n0.size * steps / (ms / 1e3) / 1e6, 1),
            'unit': 'MLUPS', 'ratio_to_headline_step': round(ms / steps / ms_headline, 4),
            'finite_density_at_end': finite, 'max_density_at_end': nmax}


def precision_table(dev, L=128, steps=5000):
    """FP32-shifted storage against the plain FP64 path on the 3D headline's
    shape at the stable coupling: D3Q19 E6, MRT rates 1.0, a droplet of radius
    L/4 (one of the headline's proportion, L*40/256, evaporates into the box at
    this size), G=-4.5, `steps` steps; errors of the density and velocity fields, of the
    mass, of the Laplace pressure (PBulk of the centre and corner densities),
    and of the spurious-current magnitude max|u|.  Two FP32 shifts: the gas
    density (the library's choice for droplets) and the mean of the two
    densities (the headline's)."""
    from sclbm.profiles import droplet
    from sclbm.sweep import laplace_dp
    box = (L, L, L)
    n0 = droplet(box, L / 4.0, RHO_L_STABLE, RHO_G_STABLE, WIDTH, SEED)
    V = n0.size
    c = L // 2
    probe = [c + L * c + L * L * c, V - 1]

    def run(prec, rho0=None):
        s = make_sim(prec, dev, box=box, g=G_STABLE, rho0=rho0)
        s.set_density(n0)
        s.set_velocity(np.zeros(3 * V))
        s.init_populations()
        m0, _ = s.reductions()
        t0 = time.perf_counter()
        s.step(steps)
        wall = time.perf_counter() - t0
        s.compute_moments()
        n, u = s.get_density(), s.get_velocity().reshape(3, -1)
        m1, _ = s.reductions()
        ni, no = s.density_at(probe)
        s.close()
        return dict(n=n, u=u, mass_drift=(m1 - m0) / m0, dp=laplace_dp(ni, no, G_STABLE)[0], n_in=ni, n_out=no,
                    umax=float(np.sqrt((u ** 2).sum(0)).max()), wall=wall)

    ref = run('fp64')
    out = {'box': list(box), 'steps': steps, 'G': G_STABLE, 'R': L / 4.0,
           'reference': 'plain FP64 GPU path (exact coefficients; within 1e-10 of the reference on the 2D twin)',
           'fp64': {'mass_drift': ref['mass_drift'], 'dp': ref['dp'], 'rho_in': ref['n_in'], 'rho_out': ref['n_out'],
                    'max_u': ref['umax'], 'wall_s': round(ref['wall'], 3)}}
    umag = np.sqrt((ref['u'] ** 2).sum(0))
    for key, rho0 in (('fp32_shift_gas', RHO_G_STABLE), ('fp32_shift_mid', 0.5 * (RHO_L_STABLE + RHO_G_STABLE))):
        r = run('fp32', rho0)
        dn = np.abs(r['n'] - ref['n'])
        du = np.sqrt(((r['u'] - ref['u']) ** 2).sum(0))
        out[key] = {'rho0': rho0,
                    'n_rel_err_max': float(dn.max() / np.abs(ref['n']).max()),
                    'n_rel_err_median': float(np.median(dn / np.abs(ref['n']))),
                    'u_err_max_over_max_u': float(du.max() / umag.max()),
                    'u_err_median_over_max_u': float(np.median(du) / umag.max()),
                    'mass_drift': r['mass_drift'],
                    'dp_rel_err': float(abs(r['dp'] - ref['dp']) / abs(ref['dp'])),
                    'rho_in_rel_err': float(abs(r['n_in'] - ref['n_in']) / ref['n_in']),
                    'rho_out_rel_err': float(abs(r['n_out'] - ref['n_out']) / ref['n_out']),
                    'max_u_rel_err': float(abs(r['umax'] - ref['umax']) / ref['umax']),
                    'wall_s': round(r['wall'], 3)}
    return out


def sweep_leg(dev, max_steps=100000, coex_steps=100000):
    """Cfg 3's ragged sweep (64 D2Q9 E8 droplets, R = 8..71) bounded for the
    default run: the batched FP32 path and the plain FP64 path droplet by
    droplet, both stopped by the same criterion (the Laplace pressure calm to
    2e-5 over 4 checks of 500 steps); wall time to converge, speed-up, and the
    Laplace-pressure error of the batch against the FP64 runs.  The plain arm
    runs the fastest FP64 arithmetic (the BGK operator factored, exact
    coefficients, FMA); the same arm with the reference's expanded operator is
    timed beside it."""
    from sclbm import sweep, _lib
    r = sweep.run_sweep(n=64, max_steps=max_steps, coex_steps=coex_steps, plain=True, device=dev,
                        plain_stop_at_dp=True, plain_literals=_lib.LIT_FACTORED,
                        plain_extra_literals=(_lib.LIT_EXACT,))
    b = r['batch']
    plain = r['plain']
    expanded = r['plain_extra'][_lib.LIT_EXACT]
    both = [j for j, p in enumerate(plain)
            if p is not None and p['status'] == 'converged' and b['status'][j] == 'converged']
    errs = np.array([abs(b['dp'][j] - plain[j]['dp']) / abs(plain[j]['dp']) for j in both])
    return {'droplets': 64, 'criterion': 'both arms: Laplace pressure calm to 2e-5 over 4 checks (500 steps apart)',
            'coexistence_wall_s': round(r['coexistence_wall_s'], 2),
            'batch_fp32': {'wall_s': round(b['wall_s'], 3),
                           'status': {str(k): int((b['status'] == k).sum()) for k in set(b['status'])},
                           'steps_max': int(np.max(b['steps']))},
            'plain_fp64': {'wall_s': round(r['plain_wall_s'], 3),
                           'arithmetic': 'FP64, BGK operator factored by opposite directions, exact coefficients, FMA',
                           'status': {k: sum(1 for p in plain if p is not None and p['status'] == k)
                                      for k in ('converged', 'max_steps', 'diverged')}},
            'speedup_wall': round(r['plain_wall_s'] / b['wall_s'], 2),
            'plain_fp64_expanded': {'wall_s': round(expanded['wall_s'], 3),
                                    'arithmetic': "FP64, the reference's expanded operator, exact coefficients, FMA",
                                    'speedup_wall': round(expanded['wall_s'] / b['wall_s'], 2)},
            'dp_rel_err_vs_fp64': {'median': float(np.median(errs)) if errs.size else None,
                                   'max': float(errs.max()) if errs.size else None,
                                   'within_1e-5': int((errs <= 1e-5).sum()), 'n': int(errs.size)},
            'unstable': len(r['unstable']),
            'not_converged_fp32': [{'R': int(b['radii'][j]), 'G': round(float(b['G'][j]), 4),
                                    'steps': int(b['steps'][j]),
                                    'fp64_steps': plain[j]['steps'] if plain[j] is not None else None}
                                   for j in range(len(b['radii'])) if b['status'][j] == 'max_steps']}


def profiled_traffic():
    """DRAM bytes per launch of the single-pass kernel from the committed ncu
    summary (captured on a smaller box and scaled by the cells it processes)."""
    p = os.path.join(ROOT, 'profiles', 'k_fused_d3q19_e6_bgk_fp32.json')
    try:
        d = json.load(open(p))
        return d['dram_bytes_per_cell'] * int(np.prod(BOX)), d
    except Exception:
        return None, None


def e2e_measure(precision, device, iters=3, lbm_steps=200, g=None, rho_l=None, rho_g=None):
    """Through the public API with host buffers: H2D of the initial density and
    velocity from pinned host memory, InitPopulations, MainLoop over lbm_steps,
    GetDensityField (D2H).  The library reads and writes the FP64 host arrays
    with a kernel where the device can reach them (pinned memory, or pageable
    memory over NVLink-C2C), else through its pinned staging buffer."""
    import torch
    from sclbm import ShanChenMultiPhase, XIStencils, FStencils, CUDA_T
    from sclbm import _lib
    from sclbm.profiles import droplet
    import sympy as sp
    ShanChenMultiPhase.verbose = False

    def pinned(a):
        t = torch.empty(a.size, dtype=torch.float64, pin_memory=True)
        out = t.numpy()
        out[:] = a.ravel()
        return out, t

    g = G if g is None else g
    rho_l = RHO_L if rho_l is None else rho_l
    rho_g = RHO_G if rho_g is None else rho_g
    n0, keep_n = pinned(droplet(BOX, R, rho_l, rho_g, WIDTH, SEED))
    u0, keep_u = pinned(np.zeros(3 * n0.size))
    res, keep_r = pinned(np.zeros(n0.size))   # the result buffer, pinned as well
    sc = ShanChenMultiPhase(lang=CUDA_T, dim_sizes=BOX, xi_stencil=XIStencils['D3Q19'],
                            f_stencil=FStencils['D3E6'], psi_code='exp(-1./ln_0)', psi_sym=None, SC_G=g,
                            tau=1.0, precision='fp32_shifted' if precision == 'fp32' else 'fp64',
                            rho0=0.5 * (rho_l + rho_g), device=device)
    pageable = sc._sim.set_transfer(_lib.TRANSFER_AUTO)
    syms = [sp.Symbol('w%d' % i) for i in range(Q)]
    mrt = dict(relaxation_matrix=sp.Matrix.diag(syms), omega_syms_vals=[(s, 1.0) for s in syms])

    def job():
        sc.sims_idpy_memory['n'].H2D(n0)
        sc.sims_idpy_memory['u'].H2D(u0)
        sc.init_status['n'] = sc.init_status['u'] = True
        sc.InitPopulations()
        sc.MainLoopMRT([0, lbm_steps], **mrt)
        return sc.GetDensityField(out=res)

    job()  # warm-up (graph capture)
    t0 = time.perf_counter()
    for _ in range(iters):
        n = job()
    dt = (time.perf_counter() - t0) / iters
    V = n0.size
    sc.End()
    return {'value': round(V * lbm_steps / dt / 1e6, 1), 'unit': 'MLUPS',
            'h2d_bytes_per_step': int(V * 8 * 4), 'd2h_bytes_per_step': int(V * 8),
            'step': 'one job: H2D rho and u (FP64 pinned host arrays, read by a kernel over the link), '
                    'InitPopulations, MainLoopMRT over %d lattice steps, GetDensityField into a pinned FP64 '
                    'result array (written by a kernel)' % lbm_steps,
            'pageable_host_access': pageable, 'G': g,
            'seconds_per_job': round(dt, 4), 'finite_density': bool(np.isfinite(n).all())}


def run_ours(a, dist):
    from sclbm.profiles import droplet
    dev = dist.local
    n0 = droplet(BOX, R, RHO_L, RHO_G, WIDTH, SEED + dist.rank)
    V = n0.size
    sim = make_sim('fp32', dev)
    sim.set_density(n0)
    sim.set_velocity(np.zeros(3 * V))
    sim.init_populations()
    # the autotuner picks the step variant (staging, tile shape, chunk) on
    # this box: each candidate timed over trial steps that leave the state as it is
    tuned, tuned_ms = sim.autotune(a.tune_steps) if a.tune_steps > 0 else (sim.get_tuning_ex(), None)
    sim.step(a.warmup)
    kps = sim.kernels_per_step()
    clocks = Clocks(dev)
    dist.barrier()
    sim.sync()
    clocks.start()
    ms = sim.step_timed(a.steps)
    ck = clocks.stop()
    dist.barrier()
    ms = dist.max(ms)
    finite, nmax = sim.density_finite()
    # per-kernel device time of the dominant kernel (events on the handle's stream)
    k_ms = sim.profile_step(20)
    path, chunk, grid = sim.get_tuning()
    sim.close()
    total = dist.ws * V * a.steps
    mlups = total / (ms / 1e3) / 1e6
    pk = peaks()
    hbm = pk['hbm_gbs'] if pk else 6800.0
    alg_bytes = 2 * Q * 4 * V                      # one read + one write of every population (FP32)
    ach = alg_bytes / (k_ms[1] / 1e3) / 1e9
    step_gbs = alg_bytes * a.steps / (ms / 1e3) / 1e9 / dist.ws * dist.ws
    out = {
        'metric': METRIC, 'value': round(mlups, 1), 'unit': 'MLUPS', 'n_gpus': dist.ws, 'steps': a.steps,
        'warmup': a.warmup, 'ms_per_step': round(ms / a.steps, 5), 'higher_is_better': True,
        'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f32', 'data': 'synthetic',
        'config': {'workload': WORKLOAD, 'box': list(BOX), 'lattice': 'D3Q19', 'stencil': 'D3E6',
                   'collision': 'MRT (rates 1.0)', 'precision': 'FP32 deviations from w_q*rho0, FP64 reductions',
                   'l2': 'inputs larger than L2 (populations 2 x %.2f GB)' % (Q * 4 * V / 1e9),
                   'parallelism': 'replicas x%d' % dist.ws if dist.ws > 1 else 'single GPU'},
        'step_path': {'path': 'single pass (k_fused, paired halo loads)' if path == 3 else
                      'single pass (k_fused)' if path == 2 else 'two passes (k_density_psi + k_fcs)',
                      'chunk_planes': chunk, 'grid': grid,
                      'tuned': dict(tuned, trial_ms_per_step=tuned_ms,
                                    tile_shape=['32x8', '64x8', '32x16', '128x8', '32x8, streaming stores',
                                                '32x8, mbarrier psi planes'][tuned.get('tile', 0)],
                                    by='sclbm_autotune (%d trial launches per candidate)' % a.tune_steps),
                      'collision_kernel': 'MRT with all rates 1.0 is exactly BGK with omega=1: sparse BGK operator'},
        'roofline': {'bound': 'hbm', 'kernel': 'k_fused (single pass)' if path in (2, 3) else
                     'k_fcs (force+collide+push-stream pass)',
                     'achieved': round(ach, 1), 'peak': hbm, 'unit': 'GB/s', 'frac': round(ach / hbm, 4),
                     'peak_source': 'MEASURED_PEAKS.json hbm_gbs (measured copy)' if pk else 'fallback 6.8 TB/s',
                     'traffic': profiled_traffic()[0], 'alg_bytes_per_launch': alg_bytes,
                     'traffic_source': (profiled_traffic()[1] or {}).get('source'),
                     'kernel_ms': round(k_ms[1], 4), 'density_pass_ms': round(k_ms[0], 4),
                     'step_alg_GBs': round(alg_bytes * a.steps / (ms / 1e3) / 1e9, 1),
                     'step_frac': round(alg_bytes * a.steps / (ms / 1e3) / 1e9 / hbm, 4)},
        'gpu_launches': int(kps * a.steps),
        'clocks': ck,
        'finite_density_at_end': finite, 'max_density_at_end': nmax,
    }
    if dist.rank == 0 and dist.ws == 1 and not a.main_only:
        # the general (dense-operator) MRT kernel, non-uniform rates, same box
        rates = np.array([1.0] * 4 + [1.2] * 6 + [1.4] * 9)
        from sclbm import _lib, XIStencils, FStencils
        x, f = XIStencils['D3Q19'], FStencils['D3E6']
        sg = _lib.Sim(3, BOX, x['XIs'], x['Ws'], x['c2'], f['Es'], f['Ws'], G, collision=_lib.COLL_MRT,
                      mrt_s=np.diag(rates), precision=_lib.FP32_SHIFTED, rho0=0.5 * (RHO_L + RHO_G), device=dev)
        sg.set_density(n0)
        sg.set_velocity(np.zeros(3 * V))
        sg.init_populations()
        sg.step(2)
        kg = max(10, a.steps // 10)
        msg = sg.step_timed(kg)
        sg.close()
        out['mrt_general'] = {'value': round(V * kg / (msg / 1e3) / 1e6, 1), 'unit': 'MLUPS', 'steps': kg,
                              'rates': 'rho,j: 1.0; stress: 1.2; higher moments: 1.4',
                              'note': 'dense population-space MRT operator (Q x Q + Q x K per cell)'}
        # plain FP64 path on the same workload (secondary): fused arithmetic with
        # exact coefficients, and the reference's arithmetic (its literals and
        # evaluation order, no FMA; GB300's FP64 rate bounds both)
        out['fp64'] = {}
        for lit, key in (('factored', 'factored_arithmetic'), ('exact', 'fused_arithmetic'),
                         ('round15', 'reference_arithmetic')):
            s64 = make_sim('fp64', dev, literals=lit)
            s64.set_density(n0)
            s64.set_velocity(np.zeros(3 * V))
            s64.init_populations()
            s64.step(2)
            k64 = max(4, a.steps // 100)
            ms64 = s64.step_timed(k64)
            kk = s64.profile_step(3)
            s64.close()
            out['fp64'][key] = {'value': round(V * k64 / (ms64 / 1e3) / 1e6, 1), 'unit': 'MLUPS', 'steps': k64,
                                'ms_per_step': round(ms64 / k64, 4),
                                'kernel_ms': [round(kk[0], 4), round(kk[1], 4)],
                                'alg_GBs': round(2 * Q * 8 * V * k64 / (ms64 / 1e3) / 1e9, 1)}
        # the fluctuating step (Gross et al. 2011) on the same box: FP32 single
        # pass with noise, MINSTD states (one generator per random moment)
        sf = make_sim('fp32', dev)
        sf.set_density(n0)
        sf.set_velocity(np.zeros(3 * V))
        sf.init_populations()
        nr, ns = _lib.noise_counts(3, Q, False)
        seeds = np.random.default_rng(SEED).integers(1, 2 ** 31 - 1, ns * V, dtype=np.uint32)
        sf.set_fluctuations('MINSTD', False, 1e-5, 1.0, seeds)
        del seeds
        sf.step(4)
        kf = max(20, a.steps // 10)
        msf = sf.step_timed(kf)
        kpf = sf.kernels_per_step()
        sf.close()
        fb = (2 * Q * 4 + 2 * nr * 4) * V                # populations + generator states, read and written
        ach_f = fb * kf / (msf / 1e3) / 1e9
        out['fluctuating'] = {'value': round(V * kf / (msf / 1e3) / 1e6, 1), 'unit': 'MLUPS', 'steps': kf,
                              'ms_per_step': round(msf / kf, 4), 'kernels_per_step': kpf,
                              'step': 'Gross 2011 fluctuating BGK (MainLoopGross2011SRT), MINSTD, kBT 1e-5, n0 1',
                              'kernel': 'k_fused_noise (single pass)' if kpf == 1 else 'k_density_psi + k_fcs_noise',
                              'alg_bytes_per_cell': (2 * Q * 4 + 2 * nr * 4),
                              'achieved_GBs': round(ach_f, 1), 'frac': round(ach_f / hbm, 4)}
        out['e2e'] = e2e_measure('fp32', dev)
        # the same job at the stable coupling: a finite result, the same cost
        out['e2e_stable'] = e2e_measure('fp32', dev, g=G_STABLE, rho_l=RHO_L_STABLE, rho_g=RHO_G_STABLE)
        out['stable_twin'] = stable_twin(dev, max(20, min(a.steps, 400)), ms / a.steps)
        if not a.no_precision:
            out['fp32_vs_fp64'] = precision_table(dev, L=a.precision_box, steps=a.precision_steps)
        if not a.no_sweep:
            out['sweep'] = sweep_leg(dev)
        if not a.no_cpu:
            out['cpu_baseline'] = cpu_measure(a.cpu_seconds)
    return out


def run_reference(a, dist):
    if dist.rank != 0:
        return None
    threads = os.cpu_count() or 1
    got = _ref_kernels('d3q19_e6_mrt1_64')
    # bounded: calibrate one step on the 64^3 sample box, then shrink the box
    # (32^3, 16^3: the same generated kernels with the box-size constants
    # re-set, as the reference sets them per box) until K+W steps fit ~150 s
    tag = 'd3q19_e6_mrt1_64'
    if got is not None:
        runner = lambda n, t: cpu_reference(n, t, tag=tag)
        dt1 = cpu_reference(1, threads, tag=tag)[1]
        for smaller in ('d3q19_e6_mrt1_32', 'd3q19_e6_mrt1_16'):
            if dt1 * (a.steps + a.warmup) <= 150.0 or _ref_kernels(smaller) is None:
                break
            tag = smaller
            dt1 = cpu_reference(1, threads, tag=tag)[1]
    else:
        runner = cpu_port
    if a.warmup:
        runner(a.warmup, threads)
    mlups, dt, V, kind = runner(a.steps, threads)
    out = {'metric': METRIC, 'value': round(mlups, 3), 'unit': 'MLUPS', 'n_gpus': dist.ws, 'steps': a.steps,
           'warmup': a.warmup, 'ms_per_step': round(dt / a.steps * 1e3, 3), 'higher_is_better': True,
           'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f64', 'data': 'synthetic', 'impl': 'reference',
           'config': {'workload': WORKLOAD + ' (CPU: %d-cell sample box per thread)' % V, 'threads': threads},
           'cpu_baseline': {'value': round(mlups, 3), 'unit': 'MLUPS', 'cores': threads, 'kind': kind,
                            'sample': '%d threads x %d steps, one independent %d-cell box each' % (
                                threads, a.steps, V)},
           'e2e': {'value': round(mlups, 3), 'unit': 'MLUPS', 'h2d_bytes_per_step': 0, 'd2h_bytes_per_step': 0}}
    return out


def run_sweep_mode(a):
    """Ragged droplet sweep (64 D2Q9 E8 droplets, R = 8..71): batched FP32 vs
    the plain FP64 path, time to converge and Laplace-pressure error; plus the
    flat-interface densities against the thermodynamic construction and a
    Laplace fit of the surface tension."""
    from sclbm import sweep
    r = sweep.run_sweep(n=a.sweep_n, max_steps=a.sweep_max_steps, plain=not a.no_plain)
    b = r['batch']
    coex = []
    for c in r['coexistence']:
        row = {k: (round(v, 6) if isinstance(v, float) else v) for k, v in c.items()}
        if c['status'] != 'diverged' and c['thermo_rho_l']:
            row['rel_dev_thermo'] = [round(c['rho_l'] / c['thermo_rho_l'] - 1, 5),
                                     round(c['rho_g'] / c['thermo_rho_g'] - 1, 5)]
        coex.append(row)
    out = {'metric': 'D2Q9 E8 droplet sweep: time to converge, batched FP32 vs plain FP64', 'unit': 's',
           'config': r['config'], 'coexistence_wall_s': round(r['coexistence_wall_s'], 2),
           'coexistence': coex, 'unstable': r['unstable'],
           'batch': {'wall_s': round(b['wall_s'], 3), 'cells': int(sum(L * L for L in b['boxes'])),
                     'status': {s: int((b['status'] == s).sum()) for s in set(b['status'])},
                     'steps_max': int(b['steps'].max()), 'steps_mean': float(b['steps'].mean())}}
    rows = []
    for j in range(len(b['radii'])):
        row = {'R': int(b['radii'][j]), 'L': int(b['boxes'][j]), 'G': round(float(b['G'][j]), 4),
               'rho_l': round(r['rho_l'][j], 6), 'rho_g': round(r['rho_g'][j], 6), 'rho_from': r['rho_source'][j],
               'steps32': int(b['steps'][j]), 'status32': str(b['status'][j]), 'dp32': float(b['dp'][j]),
               'max_u32': float(b['max_u'][j])}
        p = r['plain'][j] if 'plain' in r else None
        if p is not None:
            row.update(steps64=int(p['steps']), status64=p['status'], dp64=float(p['dp']),
                       max_u64=float(p['max_u']), wall64_s=round(p['wall_s'], 3),
                       steps64_dp_criterion=p['steps_dp'],
                       dp_rel_err=float(abs(b['dp'][j] - p['dp']) / max(abs(p['dp']), 1e-300)))
        rows.append(row)
    out['droplets'] = rows
    if 'plain' in r:
        both = [x for x in rows if x['status32'] == 'converged' and x.get('status64') == 'converged']
        errs = np.array([x['dp_rel_err'] for x in both])
        out['plain'] = {'wall_s': round(r['plain_wall_s'], 3),
                        'status': {s: sum(1 for x in rows if x.get('status64') == s) for s in
                                   set(x.get('status64') for x in rows if 'status64' in x)}}
        out['speedup_wall'] = round(r['plain_wall_s'] / b['wall_s'], 2)
        # the plain runs stopped at the batch's own criterion instead (where it fired)
        wdp = sum((p['wall_dp_s'] if p['wall_dp_s'] is not None else p['wall_s'])
                  for p in r['plain'] if p is not None)
        out['plain']['wall_same_criterion_s'] = round(wdp, 3)
        out['speedup_wall_same_criterion'] = round(wdp / b['wall_s'], 2)
        out['dp_rel_err'] = {'max': float(errs.max()) if errs.size else None,
                             'median': float(np.median(errs)) if errs.size else None,
                             'within_1e-5': int((errs <= 1e-5).sum()), 'n': int(errs.size)}
    if not a.no_laplace:
        out['laplace_fit'] = sweep.laplace_fit()
    return out


def batch_vs_plain(bres, plain):
    """Status counts, wall time and Laplace-pressure error of a batched run
    against the plain FP64 runs of the same droplets."""
    out = {'wall_s': round(bres['wall_s'], 3),
           'status': {str(k): int((bres['status'] == k).sum()) for k in set(bres['status'])},
           'steps_mean': float(np.mean(bres['steps'])), 'steps_max': int(np.max(bres['steps']))}
    if bres.get('fallback') is not None and np.isfinite(bres['residual']).any():
        res = bres['residual'][np.isfinite(bres['residual'])]
        out['warm_residual'] = {'median': float(np.median(res)), 'max': float(res.max())}
        out['cold_fallbacks'] = int(bres['fallback'].sum())
    if plain is not None:
        errs = np.array([abs(bres['dp'][j] - p['dp']) / max(abs(p['dp']), 1e-300) for j, p in enumerate(plain)
                         if p is not None and p['status'] == 'converged' and bres['status'][j] == 'converged'])
        out['dp_rel_err_vs_fp64'] = {'median': float(np.median(errs)) if errs.size else None,
                                     'max': float(errs.max()) if errs.size else None,
                                     'within_1e-5': int((errs <= 1e-5).sum()), 'n': int(errs.size)}
    return out


def run_warmstart_mode(a):
    """Learned warm start: plain-method equilibrium profiles, MLP training on
    the device, held-out evaluation, then the droplet sweep started cold and
    warm against the plain FP64 path."""
    from sclbm import sweep, warmstart
    t0 = time.perf_counter()
    prof, st = warmstart.equilibrium_profiles(n=a.ws_profiles, max_steps=a.ws_max_steps)
    train_set, test_set = warmstart.split(prof, holdout=512)
    m, loss, wall_train = warmstart.train(train_set, steps=a.ws_train_steps, batch=8192, lr=1e-3)
    ev = warmstart.evaluate(m, test_set)
    r = sweep.run_sweep(n=a.sweep_n, max_steps=a.sweep_max_steps, plain=not a.no_plain, mlp=m,
                        plain_stop_at_dp=True)
    plain = r.get('plain')
    out = {'metric': 'D2Q9 E8 droplet sweep with a learned warm start: time to converge', 'unit': 's',
           'profiles': {'requested': a.ws_profiles, 'status': st['status'], 'wall_s': round(st['wall_s'], 2),
                        'train': len(train_set), 'held_out': len(test_set),
                        'method': 'FP32 batched LBM to the Laplace-pressure criterion, radial bins of 0.5'},
           'training': {'steps': a.ws_train_steps, 'batch': 8192, 'lr': 1e-3, 'wall_s': round(wall_train, 3),
                        'loss_first': float(loss[:10].mean()), 'loss_last': float(loss[-100:].mean()),
                        'samples': int(sum(len(p['r']) for p in train_set))},
           'held_out': ev,
           'sweep': {'config': r['config'], 'coexistence_wall_s': round(r['coexistence_wall_s'], 2),
                     'unstable': len(r['unstable']),
                     'batch_cold': batch_vs_plain(r['batch'], plain),
                     'batch_warm': batch_vs_plain(r['warm'], plain)}}
    if plain is not None:
        out['sweep']['plain_fp64'] = {'wall_s': round(r['plain_wall_s'], 3),
                                      'status': {k: sum(1 for p in plain if p is not None and p['status'] == k)
                                                 for k in ('converged', 'max_steps', 'diverged')}}
        out['speedup_wall_cold'] = round(r['plain_wall_s'] / r['batch']['wall_s'], 2)
        out['speedup_wall_warm'] = round(r['plain_wall_s'] / r['warm']['wall_s'], 2)
    out['total_wall_s'] = round(time.perf_counter() - t0, 1)
    m.close()
    return out


def run_warmstart3d_mode(a):
    """Learned warm start in 3D (cfg 5): plain-method 3D equilibrium profiles
    (D3Q19 E6 droplets in 96^3 boxes), the MLP trained on them on the device,
    then the 256-droplet 3D sweep run cold and warm (cold-start fallback above
    the residual threshold) against the plain FP64 path on a timed sample, all
    arms stopped by the same Laplace-pressure criterion."""
    from sclbm import sweep, warmstart
    t0 = time.perf_counter()
    prof, st = warmstart.equilibrium_profiles_3d(n=a.ws3d_profiles, seed=11, L=96)
    train_set, test_set = warmstart.split(prof, holdout=max(8, a.ws3d_profiles // 8))
    m, loss, wall_train = warmstart.train(train_set, steps=a.ws_train_steps, batch=8192, lr=1e-3)
    ev = warmstart.evaluate(m, test_set)
    r = sweep.run_sweep3d(n=a.sweep3d_n, max_steps=a.sweep3d_max_steps, plain_sample=a.sweep3d_plain, mlp=m,
                          residual_max=0.1, plain_stop_at_dp=True)
    b, w = r['batch'], r['warm']
    ok = (b['status'] == 'converged') & (w['status'] == 'converged')
    out = {'metric': 'D3Q19 E6 droplets (96^3) with a learned warm start: time to converge', 'unit': 's',
           'profiles': {'requested': a.ws3d_profiles, 'status': st['status'], 'wall_s': round(st['wall_s'], 2),
                        'train': len(train_set), 'held_out': len(test_set)},
           'training': {'steps': a.ws_train_steps, 'wall_s': round(wall_train, 3),
                        'loss_first': float(loss[:10].mean()), 'loss_last': float(loss[-100:].mean())},
           'held_out': ev, 'config': r['config'],
           'batch_cold': {'wall_s': round(b['wall_s'], 2),
                          'status': {str(k): int((b['status'] == k).sum()) for k in set(b['status'])},
                          'steps_mean_converged': float(b['steps'][b['status'] == 'converged'].mean())},
           'batch_warm': {'wall_s': round(w['wall_s'], 2),
                          'status': {str(k): int((w['status'] == k).sum()) for k in set(w['status'])},
                          'steps_mean_converged': float(w['steps'][w['status'] == 'converged'].mean()),
                          'cold_fallbacks': int(w['fallback'].sum()),
                          'residual_median': float(np.nanmedian(w['residual']))},
           'dp_warm_vs_cold_rel': {'median': float(np.median(np.abs(w['dp'][ok] / b['dp'][ok] - 1))),
                                   'max': float(np.max(np.abs(w['dp'][ok] / b['dp'][ok] - 1)))}}
    rows = r['plain']
    if rows:
        wdp = np.mean([(p['wall_dp_s'] if p['wall_dp_s'] is not None else p['wall_s']) for p in rows])
        n_ok = int((b['status'] == 'converged').sum())
        out['plain_fp64'] = {'sample': len(rows), 'wall_per_droplet_s': round(float(wdp), 3),
                             'wall_extrapolated_s': round(float(wdp * n_ok), 1),
                             'dp_rel_err_cold': [float(abs(b['dp'][p['index']] / p['dp'] - 1)) for p in rows],
                             'dp_rel_err_warm': [float(abs(w['dp'][p['index']] / p['dp'] - 1)) for p in rows]}
        out['speedup_cold'] = round(float(wdp * n_ok / b['wall_s']), 2)
        out['speedup_warm'] = round(float(wdp * n_ok / w['wall_s']), 2)
    out['total_wall_s'] = round(time.perf_counter() - t0, 1)
    m.close()
    return out


def run_sweep3d_mode(a):
    """3D batched droplets (256 D3Q19 E6 droplets in 96^3 boxes, FP32 batches)
    against the plain FP64 path on a timed sample, extrapolated."""
    from sclbm import sweep
    from sclbm import _lib
    r = sweep.run_sweep3d(n=a.sweep3d_n, max_steps=a.sweep3d_max_steps, plain_sample=a.sweep3d_plain,
                          plain_literals=_lib.LIT_FACTORED if a.sweep3d_plain_factored else None)
    b = r['batch']
    ok = b['status'] == 'converged'
    out = {'metric': 'D3Q19 E6 batched droplets (96^3 boxes): time to converge, batched FP32 vs plain FP64',
           'unit': 's', 'config': r['config'],
           'plain_arithmetic': ('FP64, BGK operator factored, exact coefficients, FMA' if a.sweep3d_plain_factored
                                else "FP64, the reference's expanded operator, exact coefficients, FMA"),
           'batch': {'wall_s': round(b['wall_s'], 2), 'batches': b['batches'],
                     'status': {str(k): int((b['status'] == k).sum()) for k in set(b['status'])},
                     'steps_mean_converged': float(b['steps'][ok].mean()) if ok.any() else None,
                     'cell_updates': float(sum(int(st) for st in b['steps']) * r['config']['box'] ** 3)}}
    rows = []
    for p in r['plain']:
        i = p['index']
        rows.append({'R': round(float(b['radii'][i]), 3), 'G': round(float(b['G'][i]), 4), 'steps32': int(b['steps'][i]),
                     'steps64': int(p['steps']), 'status64': p['status'], 'wall64_s': round(p['wall_s'], 3),
                     'steps64_dp_criterion': p['steps_dp'],
                     'dp_rel_err': float(abs(b['dp'][i] - p['dp']) / abs(p['dp']))})
    out['plain_sample'] = rows
    if rows:
        w = np.mean([x['wall64_s'] for x in rows])
        wdp = np.mean([(p['wall_dp_s'] if p['wall_dp_s'] is not None else p['wall_s']) for p in r['plain']])
        n_ok = int(ok.sum())
        out['plain_extrapolated'] = {'wall_per_droplet_s': round(float(w), 3), 'droplets': n_ok,
                                     'wall_s': round(float(w * n_ok), 1),
                                     'wall_same_criterion_s': round(float(wdp * n_ok), 1)}
        out['speedup_wall_estimate'] = round(float(w * n_ok / b['wall_s']), 2)
        out['speedup_wall_same_criterion_estimate'] = round(float(wdp * n_ok / b['wall_s']), 2)
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument('--sweep', action='store_true', help='run the ragged droplet sweep instead')
    ap.add_argument('--sweep-n', type=int, default=64)
    ap.add_argument('--sweep-max-steps', type=int, default=100000)
    ap.add_argument('--no-plain', action='store_true')
    ap.add_argument('--no-laplace', action='store_true', help='skip the Laplace fit of the sweep mode')
    ap.add_argument('--warmstart', action='store_true', help='learned warm start: profiles, training, sweep')
    ap.add_argument('--sweep3d', action='store_true', help='3D batched droplets vs plain FP64 (sampled)')
    ap.add_argument('--sweep3d-n', type=int, default=256)
    ap.add_argument('--sweep3d-max-steps', type=int, default=20000)
    ap.add_argument('--sweep3d-plain', type=int, default=8)
    ap.add_argument('--sweep3d-plain-expanded', dest='sweep3d_plain_factored', action='store_false',
                    help="plain FP64 sample with the reference's expanded operator instead of the factored one")
    ap.add_argument('--warmstart3d', action='store_true', help='learned warm start of the 3D batched droplets')
    ap.add_argument('--ws3d-profiles', type=int, default=128)
    ap.add_argument('--ws-profiles', type=int, default=4096)
    ap.add_argument('--ws-max-steps', type=int, default=60000)
    ap.add_argument('--ws-train-steps', type=int, default=20000)
    ap.add_argument('--gpus', type=int, default=1)
    ap.add_argument('--steps', type=int, default=2000)
    ap.add_argument('--warmup', type=int, default=5)
    ap.add_argument('--impl', default='ours', choices=['ours', 'reference'])
    ap.add_argument('--cpu-seconds', type=float, default=15.0)
    ap.add_argument('--no-cpu', action='store_true')
    # profiling case: a smaller cubic box and only the main (FP32 single-pass) leg
    ap.add_argument('--box', type=int, default=0, help='cube side for a profiling run (default 256)')
    ap.add_argument('--main-only', action='store_true', help='skip the secondary legs')
    ap.add_argument('--no-precision', action='store_true', help='skip the FP32-vs-FP64 error table')
    ap.add_argument('--precision-box', type=int, default=128)
    ap.add_argument('--precision-steps', type=int, default=5000)
    ap.add_argument('--no-sweep', action='store_true', help='skip the bounded droplet-sweep leg')
    ap.add_argument('--tune-steps', type=int, default=10, help='autotuner trial launches per candidate (0: off)')
    a = ap.parse_args()
    if a.box:
        global BOX
        BOX = (a.box, a.box, a.box)
    if a.sweep:
        print(json.dumps(run_sweep_mode(a)))
        return 0
    if a.warmstart:
        print(json.dumps(run_warmstart_mode(a)))
        return 0
    if a.sweep3d:
        print(json.dumps(run_sweep3d_mode(a)))
        return 0
    if a.warmstart3d:
        print(json.dumps(run_warmstart3d_mode(a)))
        return 0
    if a.impl == 'reference':
        ws, rank, _ = dist_env()
        if rank != 0:
            return 0
        a.steps = max(1, a.steps)
        out = run_reference(a, type('D', (), {'rank': 0, 'ws': ws})())
        print(json.dumps(out))
        return 0
    dist = Dist()
    out = run_ours(a, dist)
    if dist.rank == 0:
        print(json.dumps(out))
    dist.close()
    return 0


if __name__ == '__main__':
    sys.exit(main())
