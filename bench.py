"""Benchmark of the direct-SCF J/K build on one GB300.

Workload (default --config c30): seeded synthetic 30-atom C10N3O5H12
molecule (self-avoiding random walk, 1.0-1.5 A bonds, >= 2.0 A non-bonded),
synthetic same-structure def2-TZVP basis (up to f), SAD FP64 density,
direct_scf_tol 1e-13.  One step = one J/K build for that density.

Printed JSON line (one per run, rank 0):
  value       quartets/s of the FP64 build, density and pair data resident in
              HBM, CUDA events around each build, L2 flushed between builds;
  e2e         the same metric through the public get_jk (numpy density in
              pinned host memory, host->device copy, basis transforms, build,
              device->host copy of J and K inside the timed region);
  mixed       the mixed FP32/FP64 build at split 1e-6: quartets/s, speed-up
              over FP64 and the error against the FP64 build, and a sweep
              of splits 1e-8 .. 1e-2;
  j_only      the J-only build of the same density (Coulomb-block screening);
  mixed_dense FP64 vs mixed (splits 1e-6, 1e-4) for a dense SCF density of
              the same molecule (the first SCF step from SAD), and the
              nuclear gradient of the J/K energy of that density;
  roofline    the dominant class kernel: algorithmic FP64 FLOP/s against the
              FP64 FMA peak measured here by an FMA-chain probe;
  cpu_baseline  the C++ CPU oracle on this host's cores on a bounded sample.

--impl reference runs the CPU implementation of the path (the oracle, the
restatement of PySCF's get_jk) on all host cores for the same workload.
--mode scf runs a full RHF of --config (FP64 and mixed J/K); --mode dense
times FP64 against mixed J/K on a dense SCF density of --config (c120: the
120-atom molecule); --mode grad times the nuclear gradient of the J/K
energy; --mode profile and --mode guess as their help says.
"""
import argparse
import ctypes
import json
import os
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

CONFIGS = {
    'c30': dict(formula={'C': 10, 'N': 3, 'O': 5, 'H': 12}, seed=0, basis='syn-def2-tzvp',
                workload='synthetic C10N3O5H12 (seed 0), syn-def2-tzvp, SAD density, tol 1e-13'),
    'c10': dict(formula={'C': 4, 'N': 1, 'O': 1, 'H': 4}, seed=0, basis='syn-def2-tzvp',
                workload='synthetic C4NOH4 (seed 0), syn-def2-tzvp, SAD density, tol 1e-13'),
    'c120': dict(formula={'C': 40, 'N': 8, 'O': 12, 'H': 60}, seed=0, basis='syn-def2-tzvp',
                 workload='synthetic C40N8O12H60 (seed 0), syn-def2-tzvp, RHF to 1e-8 Ha'),
    'h2o': dict(atom='O 0 0 0.1174; H -0.757 0 -0.4696; H 0.757 0 -0.4696', basis='syn-cc-pvdz',
                workload='H2O, syn-cc-pvdz, SAD density, tol 1e-13'),
}


def make_mol(cfg):
    from gpu4pyscf_gb300 import gto
    from gpu4pyscf_gb300.gto import molgen
    c = CONFIGS[cfg]
    if 'atom' in c:
        return gto.M(atom=c['atom'], basis=c['basis'])
    return molgen.make_mol(c['formula'], c['seed'], c['basis'])


def make_density(mol):
    """SAD density from the engine's own atomic SCF (GPU)."""
    from gpu4pyscf_gb300.scf import guess
    return guess.sad_density(mol)


class ClockSampler:
    """nvidia-smi clock and throttle-reason samples every 200 ms while the
    timed region runs (read only: no setting of the GPU is touched),
    summarised as the median SM clock and the reasons seen."""

    def __init__(self):
        self.proc = None
        self.path = None

    def start(self):
        try:
            import tempfile
            fd, self.path = tempfile.mkstemp(prefix='jk_clocks_', suffix='.csv')
            self.fh = os.fdopen(fd, 'w')
            self.proc = subprocess.Popen(
                ['nvidia-smi', '--query-gpu=index,clocks.sm,clocks.max.sm,power.draw,'
                 'clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,'
                 'clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,'
                 'clocks_event_reasons.sw_power_cap', '--format=csv,noheader,nounits', '-lms', '200'],
                stdout=self.fh, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
            if self.path:
                try:
                    self.fh.close()
                    os.unlink(self.path)
                except Exception:
                    pass

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        self.proc.wait()
        self.fh.close()
        sm, smax, reasons = [], None, set()
        names = ['hw_slowdown', 'hw_thermal_slowdown', 'sw_thermal_slowdown', 'sw_power_cap']
        for line in open(self.path):
            t = [x.strip() for x in line.split(',')]
            if len(t) < 9:
                continue
            try:
                sm.append(float(t[1]))
                smax = float(t[2])
            except ValueError:
                continue
            for n, v in zip(names, t[5:9]):
                if v.lower().startswith('active'):
                    reasons.add(n)
        try:
            os.unlink(self.path)
        except OSError:
            pass
        if not sm:
            return None
        return {'sm_mhz': float(np.median(sm)), 'sm_max_mhz': smax, 'reasons': sorted(reasons),
                'samples': len(sm)}


def cpu_sample(mol, dm_user, target_s=15., min_stride=1):
    """Time the C++ oracle on a bounded sample of the same J/K build: every
    stride-th bra shell pair, the stride shrunk until the sample takes a
    quarter of target_s or more (stride 1 is the whole build, whose J/K are
    returned as 'vj', 'vk' in the sorted Cartesian basis)."""
    from oracle import oracle
    from gpu4pyscf_gb300.gto.sorted_basis import SortedBasis
    sb = SortedBasis(mol)

    class Raw:
        _atm, _bas, _env = sb._atm, sb._bas, sb._env
    dms = sb.coeff @ dm_user @ sb.coeff.T
    npair = sb.nbas * (sb.nbas + 1) // 2
    cores = os.cpu_count()
    stride = max(npair // 64, min_stride, 1)
    while True:
        t0 = time.perf_counter()
        vj, vk, st = oracle.get_jk_cart(Raw, dms, hermi=1, tol=1e-13, nthreads=cores, bra_stride=stride)
        dt = time.perf_counter() - t0
        if dt > target_s / 4 or stride <= min_stride:
            break
        stride = max(min_stride, int(stride / max(2., target_s / 4 / max(dt, 1e-3))))
    return {'value': float(st[0]) / dt, 'unit': 'quartets/s', 'cores': cores, 'kind': 'port',
            'sample': 'C++ McMurchie-Davidson oracle (OpenMP, %d threads), every %d-th of %d bra shell '
                      'pairs of the same sorted basis and density: %d quartets in %.2f s'
                      % (cores, stride, npair, st[0], dt),
            'seconds': dt, 'quartets': int(st[0]), 'stride': stride,
            'vj': vj if stride == 1 else None, 'vk': vk if stride == 1 else None}


def oracle_full(mol, dm_user):
    """The oracle's whole J/K build of the benchmark density (sorted
    Cartesian basis, hermi=1, tol 1e-13) on all host cores, timed: the
    parity reference of the bench line and its CPU baseline."""
    from oracle import oracle
    from gpu4pyscf_gb300.gto.sorted_basis import SortedBasis
    sb = SortedBasis(mol)

    class Raw:
        _atm, _bas, _env = sb._atm, sb._bas, sb._env
    dms = sb.coeff @ dm_user @ sb.coeff.T
    cores = os.cpu_count()
    t0 = time.perf_counter()
    vj, vk, st = oracle.get_jk_cart(Raw, dms, hermi=1, tol=1e-13, nthreads=cores)
    dt = time.perf_counter() - t0
    base = {'value': float(st[0]) / dt, 'unit': 'quartets/s', 'cores': cores, 'kind': 'port',
            'sample': 'C++ McMurchie-Davidson oracle (OpenMP, %d threads), the whole build: every bra '
                      'shell pair of the same sorted basis and density, %d quartets in %.2f s'
                      % (cores, st[0], dt)}
    return dms, vj, vk, base


def parity_vs_oracle(vj, vk, ref_j, ref_k, dm_sorted):
    """Max |dJ|, |dK| and the two-electron energy difference of a build
    against the oracle's J/K of the same sorted density (FP64 bar: 1e-10)."""
    dj = vj - ref_j
    dk = vk - ref_k
    de = 0.5 * float(np.sum(dm_sorted * dj)) - 0.25 * float(np.sum(dm_sorted * dk))
    return {'max_abs_dJ': float(abs(dj).max()), 'max_abs_dK': float(abs(dk).max()), 'dE_2e_Ha': de}


def run_reference(args):
    rank = int(os.environ.get('RANK', '0'))
    if rank != 0:
        return
    mol = make_mol(args.config)
    dm, dm_source = reference_density(mol)
    ts = []
    for _ in range(args.warmup):
        # a short sample of the same build (thread pool, caches, pages)
        cpu_sample(mol, dm, target_s=min(4., args.ref_seconds), min_stride=8)
    res = None
    for _ in range(args.steps):
        res = cpu_sample(mol, dm, target_s=args.ref_seconds)
        ts.append(res['seconds'])
    val = res['value']
    line = {'impl': 'reference', 'metric': 'jk_quartets_per_s', 'value': val, 'unit': 'quartets/s',
            'n_gpus': args.gpus, 'steps': args.steps, 'warmup': args.warmup,
            'ms_per_step': 1e3 * float(np.mean(ts)), 'higher_is_better': True, 'scaling': 'weak',
            'vs_baseline': None, 'dtype': 'f64', 'data': 'synthetic',
            'config': {'workload': CONFIGS[args.config]['workload'], 'nao_user': mol.nao,
                       'density': dm_source},
            'cpu_baseline': {k: res[k] for k in ('value', 'unit', 'cores', 'kind', 'sample')},
            'e2e': {'value': val, 'unit': 'quartets/s', 'h2d_bytes_per_step': 0, 'd2h_bytes_per_step': 0}}
    print(json.dumps(line))


def reference_density(mol):
    """The density of the GPU arm (the engine's SAD guess) when a GPU is
    present, so both arms build J/K of the same matrix; otherwise the
    oracle's SAD, the same guess restated on the CPU."""
    try:
        import torch
        if torch.cuda.is_available():
            return make_density(mol), 'SAD (engine, as the GPU arm)'
    except Exception:  # noqa: BLE001
        pass
    from oracle import oracle
    return oracle.sad_density(mol), 'SAD (oracle restatement; no GPU)'


def fma_peak(lib, fp32):
    import torch
    out = torch.zeros(1, dtype=torch.float64, device='cuda')
    st = torch.cuda.current_stream().cuda_stream
    sm = torch.cuda.get_device_properties(0).multi_processor_count
    blocks, iters = sm * 8, 4096 if not fp32 else 65536
    lib.jk_probe_fma(out.data_ptr(), blocks, iters, fp32, st)
    torch.cuda.synchronize()
    best = 0.
    for _ in range(3):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        lib.jk_probe_fma(out.data_ptr(), blocks, iters, fp32, st)
        e1.record()
        torch.cuda.synchronize()
        t = e0.elapsed_time(e1) * 1e-3
        best = max(best, blocks * 256 * iters * 8 * 2 / t)
    return best


def make_batch(nmol=64, seed=0):
    """64 seeded molecules of 5-40 atoms (uniform count, C/N/O/H in the
    proportions of C10N3O5H12), syn-6-31g*, each with 1-4 random symmetric
    PSD densities X X^T scaled to tr(D S) = N_e."""
    import torch
    from gpu4pyscf_gb300.gto import molgen
    from gpu4pyscf_gb300.scf import hf, jk
    rng = np.random.default_rng(seed)
    mols, dms = [], []
    for m in range(nmol):
        natm = int(rng.integers(5, 41))
        mol = molgen.make_mol(molgen.formula_for(natm, rng), 1000 + m, 'syn-6-31g*')
        opt = jk._VHFOpt(mol).build()
        S, _, _ = hf.int1e_sorted(opt)
        C = opt.coeff
        S = (C.T @ S @ C).cpu().numpy()
        k = int(rng.integers(1, 5))
        x = rng.normal(size=(k, mol.nao, mol.nao))
        d = x @ x.transpose(0, 2, 1)
        for i in range(k):
            d[i] *= mol.nelectron / np.trace(d[i] @ S)
        mols.append((mol, opt))
        dms.append(d)
    return mols, dms


def run_batched(steps, warmup):
    """Batched J/K of 64 molecules: per-molecule loop vs shared class
    launches (eager) vs one CUDA-graph replay after autotuning."""
    import torch
    from gpu4pyscf_gb300.scf import jk, jk_batch
    mols, dms = make_batch()

    def timed_wall(fn, n):
        ts = []
        for _ in range(n):
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            fn()
            e1.record()
            torch.cuda.synchronize()
            ts.append(e0.elapsed_time(e1) * 1e-3)
        return float(np.median(ts))

    dms_dev = [torch.as_tensor(d, device='cuda') for d in dms]
    loop = lambda: [jk.get_jk(m, d, hermi=1, vhfopt=o) for (m, o), d in zip(mols, dms_dev)]
    for _ in range(warmup):
        loop()
    t_loop = timed_wall(loop, steps)
    b = jk_batch.BatchJK([m for m, _ in mols])
    eager = lambda: b.get_jk(dms_dev)
    for _ in range(warmup):
        eager()
    t_eager = timed_wall(eager, steps)
    b.get_jk(dms_dev, stats=True)
    nquart = b.last_stats['quartets_fp64']
    # autotune on the first 8 molecules (same classes, an eighth of the work)
    # and carry the per-class choices over to the full batch
    t0 = time.perf_counter()
    small = jk_batch.BatchJK([m for m, _ in mols[:8]])
    small.tune(dms_dev[:8], reps=1)
    b.set_variants(small.variants())
    t_tune = time.perf_counter() - t0
    for _ in range(warmup):
        eager()
    t_tuned = timed_wall(eager, steps)
    b.capture(dms_dev)
    for _ in range(warmup):
        b.replay()
    t_graph = timed_wall(b.replay, steps)
    ref = loop()
    out = b.replay()
    torch.cuda.synchronize()
    err = max(float(abs(a - r).max().item()) for a, r in zip(out[0] + out[1], [x[0] for x in ref] + [x[1] for x in ref]))
    # the whole batch in mixed precision (one launch per class and precision,
    # tuned FP64 launches), against the FP64 batch: seconds, speed-up over the
    # tuned FP64 batch, max elementwise error, max |dE_2e| over the densities
    mixed = {}
    try:
        j0, k0 = b.get_jk(dms_dev)
        for split in (1e-6, 1e-4):
            b.precision, b.split_thresh = 'mixed', split
            for _ in range(warmup):
                eager()
            t_m = timed_wall(eager, steps)
            jm, km = b.get_jk(dms_dev)
            e_max = max(float(abs(a - r).max().item()) for a, r in zip(jm + km, j0 + k0))
            de = 0.
            for d, a, a0, c, c0 in zip(dms_dev, jm, j0, km, k0):
                d3 = d if d.ndim == 3 else d[None]
                for n in range(d3.shape[0]):
                    de = max(de, abs(0.5 * float(torch.sum(d3[n] * (a[n] - a0[n])))
                                     - 0.25 * float(torch.sum(d3[n] * (c[n] - c0[n])))))
            mixed['%g' % split] = {'s_per_batch': t_m, 'speedup_vs_fp64_tuned': t_tuned / t_m,
                                   'max_abs_diff_vs_fp64': e_max, 'max_abs_dE_2e_Ha': de}
    except Exception as exc:  # noqa: BLE001
        mixed = {'error': '%s: %s' % (type(exc).__name__, exc)}
    finally:
        b.precision = 'fp64'
    return {'workload': '64 seeded C/N/O/H molecules of 5-40 atoms, syn-6-31g*, 1-4 random PSD densities each',
            'n_molecules': len(mols), 'n_densities': int(sum(d.shape[0] for d in dms)),
            'nao_total': int(sum(m.nao for m, _ in mols)), 'quartets': int(nquart),
            's_per_batch_molecule_loop': t_loop, 's_per_batch_shared_launches': t_eager,
            's_per_batch_tuned': t_tuned, 's_per_batch_graph_replay': t_graph,
            'speedup_graph_vs_loop': t_loop / t_graph, 'autotune_s': t_tune,
            'quartets_per_s_graph': nquart / t_graph, 'max_abs_diff_vs_loop': err, 'mixed': mixed}


def max_over_ranks(seconds, world, device):
    """The slowest rank's timed-region seconds (all ranks must call it)."""
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(seconds)], dtype=torch.float64, device=device)
    if world > 1:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_rate(units_per_rank, world, seconds_per_step):
    """Whole-job rate of N replicas (weak scaling: every rank does the same
    build): all ranks' units over the slowest rank's time."""
    return units_per_rank * world / seconds_per_step


def nvtx_push(name):
    try:
        import torch
        torch.cuda.nvtx.range_push(name)
    except Exception:
        pass


def nvtx_pop():
    try:
        import torch
        torch.cuda.nvtx.range_pop()
    except Exception:
        pass


def kernel_family(li, lj, lk, ll):
    """Kernel family the engine launches by default for a class: the
    register-resident kernel when the Cartesian ERI block plus one root's
    2D integrals fit in 64 registers' worth of values (LEAN_MAX in
    csrc/jk_classes.cu), else the block-cooperative one."""
    nc = lambda l: (l + 1) * (l + 2) // 2
    nf = nc(li) * nc(lj) * nc(lk) * nc(ll)
    gs = (li + 1) * (lj + 1) * (lk + 1) * (ll + 1)
    return 'rys_lean_kernel' if nf + 3 * gs <= 64 else 'rys_class_kernel'


# DRAM bytes (read + write) per launch of FP64 class kernels of the timed
# build, from one ncu capture of the c30 command (--set full, one launch of
# the class inside the 'jk_timed' NVTX range); the roofline's traffic when
# the dominant class is among them
# DRAM read + write bytes of one launch of a class, from a full ncu capture
# of that launch in this code (`--mode profile`, NVTX range jk_profile)
NCU_DRAM_BYTES = {('c30', '(11|11)'): 1685760 + 5376, ('c30', '(11|10)'): 3351808}


def train_guess_model(basis, nbase, nconf, epochs, seed=0):
    """A learned-guess network trained on this engine's converged densities
    of nbase x nconf seeded conformers (8-20 heavy atoms) in ``basis``
    (batched SCFs); returns (model, info)."""
    from gpu4pyscf_gb300.scf import learned_guess as lg
    t0 = time.perf_counter()
    confsets = lg.make_conformers(nbase, nconf, basis, seed)
    nblock = max(b - a for cs in confsets for (a, b) in lg.block_slices(cs[0]))
    data = lg.generate_batched(confsets, 0)
    t_gen = time.perf_counter() - t0
    model = lg.train(data, nblock, epochs=epochs, lr=2e-3, seed=seed)
    return model, {'basis': basis, 'train_conformers': len(data), 'generate_s': t_gen,
                   'train_s': time.perf_counter() - t0 - t_gen, 'epochs': epochs,
                   'final_train_loss': model.loss_history[-1]}


def run_scf(args):
    """Full RHF to 1e-8 Ha with DIIS on one molecule: FP64 J/K from the SAD
    guess against mixed J/K (split args.split) from the SAD guess and, with
    --guess learned, from the learned guess (a network trained first on
    converged densities of small conformers in the same basis)."""
    import torch
    from gpu4pyscf_gb300.scf import hf
    mol = make_mol(args.config)
    model, model_info = None, None
    arms = [('fp64', 'sad'), ('mixed', 'sad')]
    if args.scf_arms:
        arms = [tuple(a.split(':')) for a in args.scf_arms.split(',')]
    if args.guess == 'learned' or any(g == 'learned' for _, g in arms):
        model, model_info = train_guess_model(CONFIGS[args.config]['basis'], args.guess_bases,
                                              args.guess_conformers, args.guess_epochs)
        if ('mixed', 'learned') not in arms:
            arms.append(('mixed', 'learned'))
    rows = []
    for prec, g in arms:
        mf = hf.RHF(mol)
        mf.conv_tol = 1e-8
        mf.max_cycle = 80
        mf.precision = prec
        mf.split_thresh = args.split
        mf.verbose = True          # per-cycle progress on stderr
        print('== %s %s' % (prec, g), file=sys.stderr, flush=True)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        if g == 'learned':
            mf.init_guess, mf.guess_model = 'learned', model
        e = mf.kernel()
        torch.cuda.synchronize()
        rows.append({'precision': prec, 'guess': g, 'e_tot': e, 'cycles': mf.cycles, 'converged': mf.converged,
                     'wall_s': time.perf_counter() - t0})
    last = rows[-1]
    line = {'metric': 'scf_seconds_to_1e-8', 'value': last['wall_s'], 'unit': 's', 'n_gpus': 1,
            'higher_is_better': False, 'dtype': 'f64/mixed', 'data': 'synthetic',
            'config': {'workload': CONFIGS[args.config]['workload'], 'nao_user': mol.nao, 'natm': mol.natm,
                       'split': args.split},
            'runs': rows, 'dE_vs_first_run': [r['e_tot'] - rows[0]['e_tot'] for r in rows],
            'speedup_vs_first_run': [rows[0]['wall_s'] / r['wall_s'] for r in rows],
            'guess_model': model_info}
    print(json.dumps(line))


def run_profile(args):
    """bench.py --mode profile: the J/K build of --config (FP64, or
    --precision mixed with --split), per-class kernel times from CUDA events
    (serialised), then one more build inside the NVTX range 'jk_profile', the
    launch a profiler selects (ncu --nvtx --nvtx-include 'jk_profile/')."""
    import torch
    from gpu4pyscf_gb300.lib import libjk
    from gpu4pyscf_gb300.scf import jk
    mol = make_mol(args.config)
    dm = make_density(mol)
    opt = jk._VHFOpt(mol, direct_scf_tol=1e-13).build()
    opt.precision, opt.split_thresh = args.precision, args.split
    dms = opt.apply_coeff_C_mat_CT(torch.as_tensor(dm, device='cuda')[None]).contiguous()
    lib = libjk.load()
    opt._build(dms, 1, True, True, stats=True)
    st = dict(opt.last_stats)
    for _ in range(3):
        opt._build(dms, 1, True, True)
    ts = []
    for _ in range(5):
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        opt._build(dms, 1, True, True)
        e1.record()
        torch.cuda.synchronize()
        ts.append(e0.elapsed_time(e1))
    h = opt._handle
    lib.jk_opt_time_classes(h, 1)
    opt._build(dms, 1, True, True, stats=True)
    nq = lib.jk_n_quartet_classes()
    ms = np.zeros(2 * nq)
    fl = np.zeros(2 * nq, dtype=np.int64)
    qq = np.zeros(2 * nq, dtype=np.int64)
    L = [np.zeros(nq, dtype=np.int32) for _ in range(4)]
    best = np.full(2 * nq, np.inf)
    for _ in range(3):
        opt._build(dms, 1, True, True)
        lib.jk_opt_class_times(h, ms.ctypes.data, fl.ctypes.data, qq.ctypes.data, *[x.ctypes.data for x in L])
        best = np.minimum(best, np.where(ms > 0, ms, np.inf))
    lib.jk_opt_time_classes(h, 0)
    rows = []
    for k in range(2 * nq):
        if np.isfinite(best[k]):
            q = k // 2
            rows.append(['(%d%d|%d%d) %s' % (L[0][q], L[1][q], L[2][q], L[3][q], 'FP32' if k % 2 else 'FP64'),
                         round(float(best[k]), 4), int(qq[k]), int(fl[k]),
                         round(fl[k] / (best[k] * 1e-3) / 1e12, 4)])
    rows.sort(key=lambda r: -r[1])
    torch.cuda.synchronize()
    nvtx_push('jk_profile')
    opt._build(dms, 1, True, True)
    torch.cuda.synchronize()
    nvtx_pop()
    print(json.dumps({'mode': 'profile', 'config': CONFIGS[args.config]['workload'], 'precision': args.precision,
                      'split': args.split if args.precision != 'fp64' else None, 'build_ms': sorted(ts),
                      'stats': st, 'classes': {'columns': ['class', 'ms', 'quartets', 'model_flops', 'TFLOP/s'],
                                               'rows': rows}}))


def run_grad(args):
    """bench.py --mode grad: nuclear gradient of the J/K energy of --config
    (j_factor 1, k_factor 0.5) for the SAD density and for the dense density
    after the first SCF step, through the dedicated derivative kernels, timed
    with CUDA events (3 untimed, 5 timed), beside the route through the J/K
    kernels of the extended basis (one timed call, which builds its own
    optimizer as every call of that route does) and their agreement;
    then one more dense-density gradient inside the NVTX range
    'grad_profile'.  With --profile-only: only the dense density, one
    untimed gradient and the one in the range (the command a profiler
    runs)."""
    import torch
    from gpu4pyscf_gb300.scf import grad_jk, jk
    mol = make_mol(args.config)
    opt = jk._VHFOpt(mol, direct_scf_tol=1e-13).build()
    if args.profile_only:
        dm = dense_density(mol, host_eig=True)[0]
        grad_jk.jk_energy_grad(mol, dm, 1., .5, vhfopt=opt)
        torch.cuda.synchronize()
        nvtx_push('grad_profile')
        grad_jk.jk_energy_grad(mol, dm, 1., .5, vhfopt=opt)
        torch.cuda.synchronize()
        nvtx_pop()
        print(json.dumps({'mode': 'grad', 'profile_only': True, 'config': CONFIGS[args.config]['workload']}))
        return

    def timed(fn, n):
        ts = []
        for _ in range(n):
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            fn()
            e1.record()
            torch.cuda.synchronize()
            ts.append(e0.elapsed_time(e1) * 1e-3)
        return sorted(ts)
    dms = {'SAD': make_density(mol), 'dense': dense_density(mol)[0]}
    rows = {}
    for name, dm in dms.items():
        st = {}
        g1 = grad_jk.jk_energy_grad(mol, dm, 1., .5, vhfopt=opt, stats=st)
        for _ in range(3):
            grad_jk.jk_energy_grad(mol, dm, 1., .5, vhfopt=opt)
        t_ip1 = timed(lambda: grad_jk.jk_energy_grad(mol, dm, 1., .5, vhfopt=opt), 5)
        ext = []
        t_ext = timed(lambda: ext.append(grad_jk.jk_energy_grad(mol, dm, 1., .5, method='extended')), 1)
        g2 = ext[0]
        rows[name] = {'s_per_grad_ip1': t_ip1, 's_per_grad_extended': t_ext,
                      'speedup_ip1_vs_extended': t_ext[0] / t_ip1[0], 'quartets': st.get('quartets'),
                      'prim_quartets': st.get('prim_quartets'),
                      'quartets_per_s': st.get('quartets', 0) / t_ip1[0],
                      'prim_quartets_per_s': st.get('prim_quartets', 0) / t_ip1[0],
                      'max_abs_diff_ip1_vs_extended': (g1 - g2).abs().max().item(),
                      'max_abs_grad': g2.abs().max().item(),
                      'translational_sum': g1.sum(0).abs().max().item()}
    torch.cuda.synchronize()
    nvtx_push('grad_profile')
    grad_jk.jk_energy_grad(mol, dms['dense'], 1., .5, vhfopt=opt)
    torch.cuda.synchronize()
    nvtx_pop()
    print(json.dumps({'mode': 'grad', 'config': CONFIGS[args.config]['workload'], 'j_factor': 1., 'k_factor': .5,
                      'natm': mol.natm, 'densities': rows}))


def run_guess(args):
    """bench.py --mode guess: the learned initial guess at the scale of the
    workload (seeded conformers of 8-20 heavy-atom C/N/O/H molecules,
    syn-def2-svp; --guess-bases x --guess-conformers, the last
    --guess-holdout of each base held out), trained on the engine's
    converged FP64 densities; SCF cycles to 1e-8 Ha and energies of the
    held-out conformers from SAD and from the learned guess."""
    from gpu4pyscf_gb300.scf import learned_guess as lg
    res, _ = lg.run(args.guess_bases, args.guess_conformers, args.guess_holdout, 'syn-def2-svp',
                    args.guess_epochs, batched=True)
    res = {k: v for k, v in res.items() if k != 'rows'}
    line = {'metric': 'scf_cycles_learned_vs_sad', 'value': res['mean_cycles_learned'], 'unit': 'cycles',
            'n_gpus': 1, 'higher_is_better': False, 'dtype': 'f64 (SCF), f32 (network)', 'data': 'synthetic',
            'config': {'workload': res['workload']}, 'result': res}
    print(json.dumps(line))


def dense_density(mol, host_eig=False):
    """The density after the first SCF step from SAD (dense: what every later
    Fock build of an SCF sees), with the RHF object that made it.  host_eig:
    the generalized eigenproblem on the host (scipy) instead of torch's GPU
    eigensolver, whose library a profiler's injection can keep from
    loading."""
    import torch
    from gpu4pyscf_gb300.scf import hf
    mf = hf.RHF(mol)
    dm0 = mf.get_init_guess()
    f = mf.get_hcore() + mf.get_veff(None, dm0)
    if host_eig:
        import scipy.linalg
        e, c = scipy.linalg.eigh(f.cpu().numpy(), mf.get_ovlp().cpu().numpy())
        co = c[:, :mol.nelectron // 2]
        return torch.as_tensor(2. * co @ co.T, device='cuda'), mf
    e, c = mf.eig(f)
    return mf.make_rdm1(c, mf.get_occ(e, c)), mf


def dense_mixed(mol, splits=(1e-6, 1e-4), grad_out=None):
    """J/K of a dense SCF density of mol (the density after the first SCF
    step from SAD, what every later Fock build of an SCF sees), FP64 against
    mixed at the given splits: seconds per build (CUDA events, after one
    warm-up build each), speed-up, max |dJ|, |dK| and the two-electron energy
    change.  The SAD density of the default benchmark is block diagonal by
    atom, which the density screening exploits; this is the build of the SCF
    iterations.  grad_out (a dict): also time the nuclear gradient of the
    J/K energy of that density into it."""
    import torch
    from gpu4pyscf_gb300.scf import jk
    dm, mf = dense_density(mol)
    opt = mf.opt
    rows = []
    ref = None
    for prec, split in [('fp64', splits[0])] + [('mixed', x) for x in splits]:
        opt.precision, opt.split_thresh = prec, split
        jk.get_jk(mol, dm, 1, opt)          # warm-up (plans, workspace)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        vj, vk = jk.get_jk(mol, dm, 1, opt)
        e1.record()
        torch.cuda.synchronize()
        t = e0.elapsed_time(e1) * 1e-3
        if ref is None:
            ref = (vj, vk, t)
        de = 0.5 * float(torch.sum(dm * (vj - ref[0]))) - 0.25 * float(torch.sum(dm * (vk - ref[1])))
        rows.append({'precision': prec, 'split': split if prec != 'fp64' else None, 's_per_jk_build': t,
                     'speedup_vs_fp64': ref[2] / t, 'max_abs_dJ': float((vj - ref[0]).abs().max()),
                     'max_abs_dK': float((vk - ref[1]).abs().max()), 'dE_2e_Ha': de})
        print(json.dumps(rows[-1]), file=sys.stderr, flush=True)
    opt.precision = 'fp64'
    if grad_out is not None:
        # nuclear gradient of the J/K energy (j 1, k 0.5) of the same
        # density through the derivative kernels: one untimed, two timed
        from gpu4pyscf_gb300.scf import grad_jk
        st = {}
        g = grad_jk.jk_energy_grad(mol, dm, 1., .5, vhfopt=opt, stats=st)
        ts = []
        for _ in range(2):
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            grad_jk.jk_energy_grad(mol, dm, 1., .5, vhfopt=opt)
            e1.record()
            torch.cuda.synchronize()
            ts.append(e0.elapsed_time(e1) * 1e-3)
        grad_out.update({'s_per_grad': min(ts), 'quartets': st['quartets'], 'prim_quartets': st['prim_quartets'],
                         'prim_quartets_per_s': st['prim_quartets'] / min(ts),
                         'translational_sum': g.sum(0).abs().max().item(), 'max_abs_grad': g.abs().max().item()})
    return rows


def run_dense(args):
    """bench.py --mode dense: dense_mixed on --config, one JSON line."""
    mol = make_mol(args.config)
    rows = dense_mixed(mol)
    line = {'metric': 'jk_build_seconds_dense_density', 'value': rows[-1]['s_per_jk_build'], 'unit': 's',
            'n_gpus': 1, 'higher_is_better': False, 'dtype': 'f64/mixed', 'data': 'synthetic',
            'config': {'workload': CONFIGS[args.config]['workload'], 'nao_user': mol.nao, 'natm': mol.natm,
                       'density': 'first SCF step from SAD (dense)'},
            'runs': rows}
    print(json.dumps(line))


def run_gpu(args):
    import torch
    import torch.distributed as dist
    from gpu4pyscf_gb300.lib import libjk
    from gpu4pyscf_gb300.scf import jk

    world = int(os.environ.get('WORLD_SIZE', '1'))
    rank = int(os.environ.get('RANK', '0'))
    local = int(os.environ.get('LOCAL_RANK', '0'))
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group('nccl')
    lib = libjk.load()
    mol = make_mol(args.config)
    dm = make_density(mol)
    opt = jk._VHFOpt(mol, direct_scf_tol=1e-13).build()
    dm_dev = torch.as_tensor(dm, device='cuda')
    dms = opt.apply_coeff_C_mat_CT(dm_dev[None]).contiguous()
    nao_s = dms.shape[-1]

    # counts for the FLOP model and the quartet rate (outside the timed region)
    opt._build(dms, 1, True, True, stats=True)
    st64 = dict(opt.last_stats)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device='cuda')

    def timed(fn, steps):
        times = []
        for _ in range(steps):
            flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            fn()
            e1.record()
            torch.cuda.synchronize()
            times.append(e0.elapsed_time(e1) * 1e-3)
        return times

    build64 = lambda: opt._build(dms, 1, True, True)
    for _ in range(args.warmup):
        build64()
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    clocks = ClockSampler()
    clocks.start()
    # NVTX range: lets a profiler select the timed builds' launches
    # (ncu --nvtx --nvtx-include 'jk_timed/')
    nvtx_push('jk_timed')
    t64 = timed(build64, args.steps)
    nvtx_pop()
    clock_info = clocks.stop()
    t_step = max_over_ranks(sum(t64), world, 'cuda') / args.steps
    value = job_rate(st64['quartets_fp64'], world, t_step)

    # reference results for the error of the mixed build
    vj64, vk64 = opt._build(dms, 1, True, True)

    # mixed precision builds: the configured split, then a sweep
    dmc = dms[0]
    t64s = sum(t64) / args.steps

    mixed_results = {}

    def mixed_eval(split, prec, steps):
        opt.precision, opt.split_thresh = prec, split
        nvtx_push('jk_mixed_%g_%s' % (split, prec))
        opt._build(dms, 1, True, True, stats=True)
        nvtx_pop()
        st = dict(opt.last_stats)
        fn = lambda: opt._build(dms, 1, True, True)
        for _ in range(2):
            fn()
        tm = sum(timed(fn, steps)) / steps
        vjm, vkm = opt._build(dms, 1, True, True)
        mixed_results['mixed_%g_%s' % (split, prec)] = (vjm, vkm)
        de = float((0.5 * torch.sum(dmc * (vjm[0] - vj64[0]))
                    - 0.25 * torch.sum(dmc * (vkm[0] - vk64[0]))).item())
        opt.precision = 'fp64'
        return {'split': split, 'precision': prec,
                'value': (st['quartets_fp64'] + st['quartets_fp32']) / tm, 'unit': 'quartets/s',
                's_per_jk_build': tm, 'speedup_vs_fp64': t64s / tm,
                'quartets_fp32': st['quartets_fp32'], 'quartets_fp64': st['quartets_fp64'],
                'max_abs_dJ_sorted': float(abs(vjm - vj64).max().item()),
                'max_abs_dK_sorted': float(abs(vkm - vk64).max().item()),
                'dE_2e_Ha': de}

    mixed = mixed_eval(args.split, 'mixed', args.steps)
    sweep = []
    for split in (1e-8, 1e-6, 1e-4, 1e-3, 1e-2):
        for prec in ('mixed', 'mixed-fp32roots'):
            r = mixed_eval(split, prec, 2)
            if split not in (1e-8, 1e-6):
                mixed_results.pop('mixed_%g_%s' % (split, prec), None)
            sweep.append([split, prec, round(r['s_per_jk_build'], 5), round(r['speedup_vs_fp64'], 3),
                          r['max_abs_dJ_sorted'], r['max_abs_dK_sorted'], r['dE_2e_Ha']])
    mixed['sweep'] = {'columns': ['split', 'precision', 's_per_jk_build', 'speedup_vs_fp64',
                                  'max_abs_dJ', 'max_abs_dK', 'dE_2e_Ha'], 'rows': sweep}

    # J-only build of the same density: the J engine's screening (the
    # Coulomb blocks D_ij, D_kl only) on the same kernels with K off;
    # reported, never fatal to the line
    try:
        opt._build(dms, 1, True, False, stats=True)
        stj = dict(opt.last_stats)
        build_j = lambda: opt._build(dms, 1, True, False)
        for _ in range(2):
            build_j()
        tj = sum(timed(build_j, args.steps)) / args.steps
        vjj, _ = opt._build(dms, 1, True, False)
        j_only = {'s_per_j_build': tj, 'quartets': stj['quartets_fp64'],
                  'quartets_per_s': stj['quartets_fp64'] / tj, 'speedup_vs_jk_build': t64s / tj,
                  'max_abs_dJ_vs_jk_build': float(abs(vjj[0] - vj64[0]).max().item())}
    except Exception as exc:  # noqa: BLE001
        j_only = {'error': '%s: %s' % (type(exc).__name__, exc)}

    # per-class kernel times (CUDA events on the build stream) for the roofline
    h = opt._handle
    lib.jk_opt_time_classes(h, 1)
    opt._build(dms, 1, True, True, stats=True)
    torch.cuda.synchronize()
    nq = lib.jk_n_quartet_classes()
    ms = np.zeros(2 * nq)
    fl = np.zeros(2 * nq, dtype=np.int64)
    qq = np.zeros(2 * nq, dtype=np.int64)
    L = [np.zeros(nq, dtype=np.int32) for _ in range(4)]
    best_ms = np.full(2 * nq, np.inf)
    for _ in range(3):
        flush.zero_()
        opt._build(dms, 1, True, True)
        lib.jk_opt_class_times(h, ms.ctypes.data, fl.ctypes.data, qq.ctypes.data,
                               *[x.ctypes.data for x in L])
        best_ms = np.minimum(best_ms, np.where(ms > 0, ms, np.inf))
    # the same for the mixed build: FP32 class kernels (odd slots)
    opt.precision, opt.split_thresh = 'mixed', args.split
    opt._build(dms, 1, True, True, stats=True)
    ms32 = np.full(2 * nq, np.inf)
    fl32 = np.zeros(2 * nq, dtype=np.int64)
    qq32 = np.zeros(2 * nq, dtype=np.int64)
    for _ in range(2):
        flush.zero_()
        opt._build(dms, 1, True, True)
        lib.jk_opt_class_times(h, ms.ctypes.data, fl32.ctypes.data, qq32.ctypes.data,
                               *[x.ctypes.data for x in L])
        ms32 = np.minimum(ms32, np.where(ms > 0, ms, np.inf))
    ms32[~np.isfinite(ms32)] = 0.
    opt.precision = 'fp64'
    lib.jk_opt_time_classes(h, 0)
    fp32_classes = []
    for q in range(nq):
        if ms32[2 * q + 1] > 0:
            fp32_classes.append(['(%d%d|%d%d)' % (L[0][q], L[1][q], L[2][q], L[3][q]),
                                 round(float(ms32[2 * q + 1]), 4), int(qq32[2 * q + 1]),
                                 round(float(ms32[2 * q]), 4), int(qq32[2 * q])])
    fp32_classes.sort(key=lambda r: -r[1])
    mixed['classes_top_fp32'] = fp32_classes[:8]
    mixed['sum_fp32_class_ms'] = float(ms32[1::2].sum())
    mixed['sum_fp64_class_ms'] = float(ms32[0::2].sum())
    best_ms[~np.isfinite(best_ms)] = 0.
    k = int(np.argmax(best_ms[0::2])) * 2
    peak64 = fma_peak(lib, 0)
    peak32 = fma_peak(lib, 1)
    dom = {'class': '(%d%d|%d%d)' % (L[0][k // 2], L[1][k // 2], L[2][k // 2], L[3][k // 2]),
           'ms': float(best_ms[k]), 'flops': int(fl[k]), 'quartets': int(qq[k]),
           'share_of_build': float(best_ms[k] / max(best_ms[0::2].sum(), 1e-12))}
    achieved = fl[k] / (best_ms[k] * 1e-3) / 1e12 if best_ms[k] > 0 else 0.
    total_fp64_tflops = st64['flops_fp64'] / t_step / 1e12
    lk4 = tuple(int(L[i][k // 2]) for i in range(4))
    traffic = NCU_DRAM_BYTES.get((args.config, dom['class']))
    roofline = {'bound': 'fp64', 'achieved': achieved, 'peak': peak64 / 1e12, 'unit': 'TFLOP/s',
                'frac': achieved / (peak64 / 1e12), 'traffic': traffic,
                'traffic_source': ('DRAM read + write of one launch of this class from a full ncu capture '
                                   'of bench.py --mode profile (same code), not measured in this '
                                   'run' if traffic else None),
                'kernel': '%s %s FP64' % (kernel_family(*lk4), dom['class']), 'dominant': dom,
                'peak_source': 'FP64 FMA-chain probe measured in this run (MEASURED_PEAKS.json has no FP64 figure)',
                'fp32_peak_tflops': peak32 / 1e12,
                'whole_build_fp64_tflops': total_fp64_tflops,
                'whole_build_frac': total_fp64_tflops / (peak64 / 1e12)}
    per_class = []
    for q in range(nq):
        if best_ms[2 * q] > 0:
            per_class.append(['(%d%d|%d%d)' % (L[0][q], L[1][q], L[2][q], L[3][q]),
                              round(float(best_ms[2 * q]), 4), int(qq[2 * q]), int(fl[2 * q])])
    per_class.sort(key=lambda r: -r[1])

    # end to end through the public API
    dm_host = torch.from_numpy(np.ascontiguousarray(dm)).pin_memory()
    out_j = torch.empty_like(dm_host).pin_memory()
    out_k = torch.empty_like(dm_host).pin_memory()

    def e2e():
        d = dm_host.to('cuda', non_blocking=True)
        vj, vk = jk.get_jk(mol, d, hermi=1, vhfopt=opt)
        out_j.copy_(vj, non_blocking=True)
        out_k.copy_(vk, non_blocking=True)

    for _ in range(args.warmup):
        e2e()
    if world > 1:
        dist.barrier()
    te = timed(e2e, args.steps)
    e2e_val = job_rate(st64['quartets_fp64'], world, max_over_ranks(sum(te), world, 'cuda') / args.steps)
    nbytes = dm_host.numel() * 8

    batched = None
    if not args.no_batch:
        batched = run_batched(2, 1)

    # mixed precision on the density an SCF iteration sees (dense), next to
    # the SAD-density numbers above; reported, never fatal to the line
    grad_dense = {'what': 'nuclear gradient of the J/K energy (j 1, k 0.5) of the same dense density, '
                          'derivative kernels (jk_energy_grad)'}
    try:
        mixed_dense = {'density': 'first SCF step from SAD (dense)', 'runs': dense_mixed(mol, grad_out=grad_dense)}
        mixed_dense['grad'] = grad_dense
    except Exception as exc:  # noqa: BLE001
        mixed_dense = {'error': '%s: %s' % (type(exc).__name__, exc)}

    # the oracle's whole build of the same density: parity of the FP64 and
    # mixed builds, and the CPU baseline (rank 0, N=1); configurations whose
    # whole oracle build would take minutes fall back to a strided sample
    # and report no parity
    cpu, parity = None, None
    if rank == 0 and world == 1 and not args.no_cpu:
        if args.config in ('c30', 'c10', 'h2o'):
            dm_s, ref_j, ref_k, cpu = oracle_full(mol, dm)
            parity = {'vs': 'oracle (C++ McMurchie-Davidson, tol 1e-13), same sorted density',
                      'tolerance_fp64': 1e-10, 'tolerance_mixed_elementwise': 1e-7,
                      'fp64': parity_vs_oracle(vj64[0].cpu().numpy(), vk64[0].cpu().numpy(), ref_j, ref_k, dm_s)}
            for key, (vjm, vkm) in mixed_results.items():
                parity[key] = parity_vs_oracle(vjm[0].cpu().numpy(), vkm[0].cpu().numpy(), ref_j, ref_k, dm_s)
        else:
            cpu = cpu_sample(mol, dm, target_s=args.cpu_seconds)
            cpu = {k: cpu[k] for k in ('value', 'unit', 'cores', 'kind', 'sample')}

    if rank == 0:
        line = {'metric': 'jk_quartets_per_s', 'value': value, 'unit': 'quartets/s', 'n_gpus': world,
                'steps': args.steps, 'warmup': args.warmup, 'ms_per_step': 1e3 * t_step,
                'higher_is_better': True, 'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f64',
                'data': 'synthetic',
                'config': {'workload': CONFIGS[args.config]['workload'], 'nao_user': mol.nao,
                           'nao_sorted_cart': nao_s, 'n_dm': 1, 'l2': 'flushed (256 MiB write) between steps',
                           'parallelism': 'replicas' if world > 1 else 'single GPU'},
                's_per_jk_build': t_step, 'quartets_per_build': st64['quartets_fp64'],
                'prim_quartets_per_build': st64['prim_quartets_fp64'],
                'fp64_tflops_model': total_fp64_tflops,
                'e2e': {'value': e2e_val, 'unit': 'quartets/s', 'h2d_bytes_per_step': nbytes,
                        'd2h_bytes_per_step': 2 * nbytes, 's_per_step': sum(te) / args.steps},
                'gpu_launches': int(st64['kernel_launches']) * args.steps,
                'mixed': mixed, 'j_only': j_only, 'mixed_dense': mixed_dense, 'roofline': roofline, 'classes_top': per_class[:8],
                'batched': batched, 'cpu_baseline': cpu, 'parity': parity, 'clocks': clock_info}
        print(json.dumps(line))
    if world > 1:
        dist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument('--gpus', type=int, default=1)
    ap.add_argument('--steps', type=int, default=5)
    ap.add_argument('--warmup', type=int, default=3)
    ap.add_argument('--impl', default='gb300', choices=['gb300', 'reference'])
    ap.add_argument('--config', default='c30', choices=sorted(CONFIGS))
    ap.add_argument('--split', type=float, default=1e-6)
    ap.add_argument('--cpu-seconds', type=float, default=15.)
    ap.add_argument('--ref-seconds', type=float, default=20.)
    ap.add_argument('--no-cpu', action='store_true')
    ap.add_argument('--no-batch', action='store_true')
    ap.add_argument('--precision', default='fp64', choices=['fp64', 'mixed', 'mixed-fp32roots'],
                    help='--mode profile: precision of the profiled build')
    ap.add_argument('--mode', default='jk', choices=['jk', 'scf', 'dense', 'guess', 'profile', 'grad'],
                    help='jk: the J/K benchmark line; scf: full RHF of --config (e.g. c120); '
                         'dense: FP64 vs mixed J/K of a dense SCF density of --config; '
                         'guess: the learned initial guess against SAD; '
                         'profile: per-class times and one build in the NVTX range jk_profile; '
                         'grad: nuclear gradient of the J/K energy (derivative kernels)')
    ap.add_argument('--profile-only', action='store_true',
                    help='--mode grad: only the gradient inside the NVTX range grad_profile')
    ap.add_argument('--guess', default='sad', choices=['sad', 'learned'],
                    help='--mode scf: add a mixed-precision run from the learned guess')
    ap.add_argument('--scf-arms', default=None,
                    help='--mode scf: comma list of precision:guess runs (default fp64:sad,mixed:sad)')
    ap.add_argument('--guess-bases', type=int, default=40)
    ap.add_argument('--guess-conformers', type=int, default=50)
    ap.add_argument('--guess-holdout', type=int, default=5)
    ap.add_argument('--guess-epochs', type=int, default=200)
    args = ap.parse_args()
    if args.impl == 'reference':
        run_reference(args)
    elif args.mode == 'scf':
        run_scf(args)
    elif args.mode == 'dense':
        run_dense(args)
    elif args.mode == 'guess':
        run_guess(args)
    elif args.mode == 'profile':
        run_profile(args)
    elif args.mode == 'grad':
        run_grad(args)
    else:
        run_gpu(args)


if __name__ == '__main__':
    main()
