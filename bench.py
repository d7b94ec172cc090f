"""Benchmark of the DUGKS time step on GB300.

Workloads (--workload):
  rt8192 (default)  large Allen-Cahn Rayleigh-Taylor: 8192x8192 cells, bounce-back
                    walls top/bottom, periodic sides, D2Q9 HCZ flow + D2Q9 Allen-Cahn
                    phase field, Atwood 0.5, Re = 10000, single-mode cosine interface
                    at mid-height (amplitude 0.05 L) plus seeded 1e-4 white noise on
                    phi; FP32 deviation storage, with the plain FP64 path timed on the
                    same grid and the per-field FP32-vs-FP64 error reported
  rt512x2048        Rayleigh-Taylor 512x2048 cells, Re = 3000, interface at y = 2L
                    (amplitude 0.1 L); plain FP64 by default
One "step" is one DUGKS time step over all cells; the metric is cell updates
per second (MLUPS), with the fused step's HBM traffic against the measured peak.

Arms:
  (default)          this library through its C ABI; state resident in HBM
  --impl reference   the CPU restatement of the reference solver (the
                     reference's own C++ cannot be built on the GPU machine),
                     all host threads, a bounded sample
One JSON line is printed by rank 0.  Multi-GPU: one process per GPU, each a
full independent replica of the workload (weak scaling, no collective).
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

SQRT_GL = 0.04                  # sqrt(g L) in lattice units (low-Mach gravity wave speed)
RHO_H, RHO_L = 3.0, 1.0         # Atwood (3-1)/(3+1) = 0.5

WORKLOADS = {
    'rt8192': dict(nx=8192, ny=8192, re=10000.0, init=[0.5, 0.05, 1e-4], precision='fp32dev',
                   name='rayleigh_taylor_8192x8192_hcz_walls', full_steps=10000, yc=0.5),
    'rt512x2048': dict(nx=512, ny=2048, re=3000.0, init=[], precision='fp64',
                       name='rayleigh_taylor_512x2048_hcz_walls', full_steps=20000, yc=2.0),
}

# algorithmic HBM bytes per cell and step: the compulsory state, read once and written once
#   FP32 storage, Allen-Cahn D2Q9: 18 distributions + 2 aux (prev phi u, v), 4 B each = 160 B
#   FP64 (multi-kernel step): 18 distributions + 2 aux planes, 8 B each = 320 B
ALGO_BYTES = {'fp32dev': 160, 'fp64': 320, 'fp64fma': 320, 'fp64fused': 320}
# bytes the FP32 step actually stores per cell and step: a state copy is 25 FP32 planes
# (9 f, 8 phase-field remainders, the phi pair, 6 aux: the force and density gradient
# are kept rather than recomputed), read and written
STORED_BYTES = {'fp32dev': 200, 'fp64': 320, 'fp64fma': 320, 'fp64fused': 400}
# DRAM bytes per cell and step of the fused FP32 kernel: ncu dram__bytes_read.sum +
# dram__bytes_write.sum of one k_stream32 launch on 3072x3072 cells, divided by the cells
# (profiles/k_stream32_rt3072x3072_fp32.md); scaled by the cell count to a full launch
TRAFFIC_BYTES = {'fp32dev': (995.413248e6 + 902.451712e6) / (3072 * 3072)}


def case_kw(wl: dict) -> dict:
    L = wl['nx']
    return dict(Mu0=SQRT_GL * L / wl['re'], M_Phi=0.02, W=4.0, Sigma=5e-5, RhoL=RHO_H, RhoV=RHO_L,
                Gy=SQRT_GL ** 2 / L)


def env_dist():
    rank = int(os.environ.get('RANK', 0))
    world = int(os.environ.get('WORLD_SIZE', 1))
    local = int(os.environ.get('LOCAL_RANK', 0))
    return rank, world, local


def load_peaks():
    p = ROOT / 'MEASURED_PEAKS.json'
    if p.exists():
        d = json.loads(p.read_text())
        return float(d.get('hbm_gbs', 6800.0)), 'measured'
    return 6800.0, 'fallback'


def fp64_peak_tflops(n: int = 4096, reps: int = 5) -> float:
    """FP64 throughput this GPU reaches in a library GEMM (torch float64 matmul, cuBLAS
    DGEMM, 2 n^3 flops), best of `reps`: the denominator of the FP64 path's %FP64."""
    import torch
    a = torch.randn(n, n, dtype=torch.float64, device='cuda')
    b = torch.randn(n, n, dtype=torch.float64, device='cuda')
    torch.matmul(a, b)
    torch.cuda.synchronize()
    best = float('inf')
    for _ in range(reps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.matmul(a, b)
        e1.record()
        torch.cuda.synchronize()
        best = min(best, e0.elapsed_time(e1))
    return 2.0 * n ** 3 / (best * 1e-3) / 1e12


def fp64_pipe(lups: float) -> dict:
    """The plain FP64 step against the FP64 rate a library GEMM reaches on this GPU."""
    peak = fp64_peak_tflops()
    out = {'peak_tflops': round(peak, 4), 'peak_source': 'measured: torch float64 matmul 4096^3 (cuBLAS DGEMM)'}
    if FP64_FLOPS_PER_CELL:
        ach = FP64_FLOPS_PER_CELL * lups / 1e12
        # a DGEMM issues DFMAs only (2 flops each): its instruction rate is peak / 2
        instr = FP64_INSTR_PER_CELL * lups / 1e12
        out.update({'flops_per_cell': FP64_FLOPS_PER_CELL, 'achieved_tflops': round(ach, 4),
                    'frac': round(ach / peak, 4), 'instr_per_cell': FP64_INSTR_PER_CELL,
                    'instr_frac': round(instr / (peak / 2), 4)})
    return out


# FP64 operations per cell-update of the plain FP64 step (k_collide + k_faces_ac + k_update
# on the 512x2048 Rayleigh-Taylor case, reference-exact variant): ncu counts of the DADD,
# DMUL and DFMA thread instructions of one step divided by the cells, a DFMA counted as two
# (profiles/fp64_step_rt512x2048_fp64_ops.md)
FP64_FLOPS_PER_CELL = 1720
FP64_INSTR_PER_CELL = 1620


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""

    QUERY = ('index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,'
             'clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,'
             'clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap')

    def __init__(self, gpu_index: int):
        self.idx = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(['nvidia-smi', f'--id={self.idx}', f'--query-gpu={self.QUERY}',
                                          '--format=csv,noheader,nounits', '-lms', '200'],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ['hw_slowdown', 'hw_thermal_slowdown', 'sw_thermal_slowdown', 'sw_power_cap']
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(',')]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for k, nm in enumerate(names):
                if parts[5 + k].lower().startswith('active'):
                    reasons.add(nm)
        if not sm:
            return {'sm_mhz': None, 'sm_max_mhz': mx, 'reasons': sorted(reasons), 'samples': 0}
        return {'sm_mhz': statistics.median(sm), 'sm_max_mhz': mx, 'reasons': sorted(reasons),
                'samples': len(sm)}


# ---------------------------------------------------------------- CPU restatement

CPU_SAMPLE = (512, 2048)  # cells of the bounded CPU sample (Rayleigh-Taylor, interface at y = 2L)


def cpu_sample(wl: dict, steps: int, threads: int):
    """The CPU restatement of the reference step on a bounded sample of the workload:
    the same case constants on a 512x2048 Rayleigh-Taylor grid (the per-cell work of
    the step does not depend on the grid size)."""
    from oracle.oracle import Oracle
    nx, ny = CPU_SAMPLE if wl['nx'] * wl['ny'] > CPU_SAMPLE[0] * CPU_SAMPLE[1] else (wl['nx'], wl['ny'])
    o = Oracle('HCZ', nx, ny, True, 'ac_rt', **case_kw(wl))
    o.step(1, threads)  # first-touch / warm-up
    t0 = time.perf_counter()
    o.step(steps, threads)
    dt = time.perf_counter() - t0
    return nx * ny * steps / dt / 1e6, dt, (nx, ny)


def cpu_baseline(wl: dict, seconds: float, fixed_steps: int = 0):
    thr = os.cpu_count() or 1
    _, one, _ = cpu_sample(wl, 1, thr)
    nsteps = fixed_steps or max(2, int(seconds / max(one, 1e-3)))
    mlups, secs, (nx, ny) = cpu_sample(wl, nsteps, thr)
    out = {'value': round(mlups, 4), 'unit': 'MLUPS', 'cores': thr, 'kind': 'port',
           'sample': f'{nsteps} steps of a {nx}x{ny} Rayleigh-Taylor grid with the case constants of '
                     f'{wl["name"]} on the CPU restatement (OpenMP, {thr} threads, {secs:.1f} s)'}
    # the unmodified reference against the restatement on the same cores, where the reference
    # builds (oracle/ref/time_reference.py): the restatement's speed over the reference's
    cal = ROOT / 'oracle' / 'ref' / 'reference_timing.json'
    if cal.exists():
        out['reference_calibration'] = json.loads(cal.read_text())
    return out, nsteps, secs


def run_reference(args, wl, rank, world):
    """The reference arm: the CPU restatement of the reference step on all host cores.
    Each of the W untimed and K timed steps is one step of the same physics on a
    bounded sample of the workload (the Rayleigh-Taylor case constants on a grid of
    2048 rows and up to 512 columns, narrowed so that the W + K steps take about three
    minutes at most); value = sampled cell updates over the K timed steps."""
    if rank != 0:
        return 0
    from oracle.oracle import Oracle
    thr = os.cpu_count() or 1
    ny = min(wl['ny'], CPU_SAMPLE[1])
    nx = min(wl['nx'], CPU_SAMPLE[0])
    o = Oracle('HCZ', nx, ny, True, 'ac_rt', **case_kw(wl))
    t0 = time.perf_counter()
    o.step(1, thr)  # first touch; its time sizes the sample
    one = time.perf_counter() - t0
    budget = 180.0
    if one * (args.steps + args.warmup) > budget:
        nx = max(32, int(nx * budget / (one * (args.steps + args.warmup))) // 32 * 32)
        o = Oracle('HCZ', nx, ny, True, 'ac_rt', **case_kw(wl))
        o.step(1, thr)
    o.step(args.warmup, thr)
    t0 = time.perf_counter()
    o.step(args.steps, thr)
    secs = time.perf_counter() - t0
    mlups = nx * ny * args.steps / secs / 1e6
    cpu = {'value': round(mlups, 4), 'unit': 'MLUPS', 'cores': thr, 'kind': 'port',
           'sample': f'each step: one step of a {nx}x{ny} Rayleigh-Taylor grid with the case constants of '
                     f'{wl["name"]} on the CPU restatement (OpenMP, {thr} threads); {args.steps} timed steps '
                     f'in {secs:.1f} s after {args.warmup} warm-up steps [reference arm]'}
    line = {
        'impl': 'reference', 'metric': 'MLUPS', 'value': cpu['value'], 'unit': 'MLUPS', 'n_gpus': world,
        'steps': args.steps, 'warmup': args.warmup, 'ms_per_step': round(1e3 * secs / max(args.steps, 1), 4),
        'higher_is_better': True, 'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f64',
        'data': 'synthetic (seeded Rayleigh-Taylor initial condition, no dataset)',
        'config': {'workload': wl['name'], 'cells': wl['nx'] * wl['ny'], 'l2_flush': 'n/a (CPU)',
                   'sample_cells_per_step': nx * ny},
        'cpu_baseline': cpu,
        'e2e': {'value': cpu['value'], 'unit': 'MLUPS', 'h2d_bytes_per_step': 0, 'd2h_bytes_per_step': 0},
    }
    print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------- serving stream

SERVING = dict(cases=256, rate=20.0, median_n=256, sigma_ln=0.6931471805599453, n_min=64, n_max=1024,
               steps=5000, ac_share=0.7, seed=2026)


def serving_stream(cases: int, steps: int, seed: int):
    """The seeded serving workload: Poisson arrivals (mean 20/s), N ~ lognormal
    (median 256, sigma_ln = ln 4 / 2) clipped to [64, 1024], 70% Allen-Cahn
    droplets / bubbles (R = N/5, density ratio U[2, 100], sigma U[1e-4, 1e-2])
    and 30% pseudopotential D2V16 cases (T/Tc U[0.6, 0.85], Carnahan-Starling
    a = 0.5, b = 4, R = 1, seeded density noise rho_c (1 + 0.01 U(-1, 1))), all
    in FP32 storage."""
    import numpy as np
    rng = np.random.default_rng(seed)
    t = np.cumsum(rng.exponential(1.0 / SERVING['rate'], cases))
    n = np.clip(np.round(SERVING['median_n'] * np.exp(rng.normal(0.0, np.log(4.0) / 2, cases))),
                SERVING['n_min'], SERVING['n_max']).astype(int)
    kind = rng.random(cases) < SERVING['ac_share']
    ratio = rng.uniform(2.0, 100.0, cases)
    sigma = rng.uniform(1e-4, 1e-2, cases)
    bubble = rng.random(cases) < 0.5
    tr = rng.uniform(0.6, 0.85, cases)
    out = []
    for k in range(cases):
        if kind[k]:
            out.append(dict(model='AC', t=float(t[k]), n=int(n[k]), rho_v=float(1.0 / ratio[k]),
                            sigma=float(sigma[k]), init='ac_drop' if bubble[k] else 'ac_drop_inside',
                            params=[float(n[k]) / 5.0], steps=steps))
        else:
            out.append(dict(model='PP16', t=float(t[k]), n=int(n[k]), tr=float(tr[k]), init='pp_noise',
                            params=[PP_RHO_C, 0.01], steps=steps))
    return out


# Carnahan-Starling with a = 0.5, b = 4, R = 1 (the EOS of Ark/Lib/nonidealEoS.h, whose b is 4):
# Tc = 0.3773 a / (b R), rho_c = 0.5218 / b (eta_c = b rho_c / 4 = 0.13044)
PP_A, PP_TC, PP_RHO_C = 0.5, 0.3773 * 0.5 / 4.0, 0.13044
# D2V16 lattice speed and viscosity of the pseudopotential cases.  The reference's
# c = 1.2 is linearly unstable for relaxation times above ~0.3 (oracle/d2v16_stability.py),
# which a vapour phase (nu = Mu0 / rho) always reaches; c = 0.5 is stable for nu from
# 0.01 to 10.  Mu0 is not given by the configurations: 0.3 keeps the spurious currents of
# the separated phases (~0.1 at T = 0.7 Tc) finite, where 0.03 and 1.0 diverge.
D2V16_C, PP_MU0 = 0.5, 0.3
# the pseudopotential cases are checked every 1000 steps, like the Allen-Cahn cases
# (the reference's residual cadence)
PP_CHECK_EVERY = 1000


def serving_case(c: dict, precision: str):
    from mpdugks_gb300 import capi
    if c['model'] == 'PP16':
        return capi.make_case('PP16', precision, Tr=c['tr'], aCS=PP_A, Tc_CS=PP_TC, d2v16_c=D2V16_C, Mu0=PP_MU0)
    return capi.make_case('AC', precision, Mu0=0.02, M_Phi=0.02, W=4.0, Sigma=c['sigma'], RhoL=1.0,
                          RhoV=c['rho_v'])


def serving_bench(args) -> dict:
    """Cases arrive on their schedule and are submitted to the server as they
    arrive; p50/p99 time to solution (submit to result on the host) and the
    aggregate rate.  Every case is checked every 1000 steps (the reference's
    residual control): a non-finite state stops it.  Beside it: the same work one
    case at a time (FP64 plain path, and FP32 storage without batching), timed on a
    sample of each model's cases, as cases/s."""
    import numpy as np
    import torch
    from mpdugks_gb300 import capi
    stream = serving_stream(args.serving_cases, args.serving_steps, SERVING['seed'])
    ac = [c for c in stream if c['model'] == 'AC']

    def serve(paced: bool):
        srv = capi.Server()
        t0 = time.perf_counter()
        ids = []
        for c in stream:
            dt = c['t'] - (time.perf_counter() - t0)
            if paced and dt > 0:
                time.sleep(dt)
            ids.append(srv.submit(serving_case(c, 'fp32dev'), c['n'], c['n'], False, c['init'], c['params'],
                                  nsteps=c['steps'], check_every=PP_CHECK_EVERY if c['model'] == 'PP16' else 0))
        tts, finite, lu, ran = [], 0, 0, []
        t_first, t_last = None, 0.0
        pp = {'submitted': 0, 'completed': 0, 'diverged': 0, 'failed': 0, 'steps_at_stop': [], 'tts': []}
        for cid, c in zip(ids, stream):
            st = srv.wait(cid, 3600.0)
            ran.append(int(st.steps_done))
            t_first = st.t_submit if t_first is None else min(t_first, st.t_submit)
            t_last = max(t_last, st.t_done)
            if c['model'] == 'PP16':
                pp['submitted'] += 1
                pp['completed'] += int(st.state == 2)
                pp['diverged'] += int(st.stop_reason == 2)
                pp['failed'] += int(st.state == 4)
                pp['steps_at_stop'].append(int(st.steps_done))
                pp['tts'].append(st.t_done - st.t_submit)
                srv.release(cid)
                continue
            if st.state != 2:
                continue
            r = srv.result(cid)
            finite += int(np.isfinite(r['rho']).all())
            srv.release(cid)
            tts.append(st.t_done - st.t_submit)
            lu += c['n'] * c['n'] * c['steps']
        stats = srv.stats()
        srv.close()
        steps = pp.pop('steps_at_stop')
        ptts = pp.pop('tts')
        if steps:
            pp['steps_at_stop_min_max'] = [min(steps), max(steps)]
            pp['tts_p50_s'] = round(float(np.percentile(ptts, 50)), 4)
        return tts, finite, lu, t_last - (t_first or 0.0), stats, pp, ran

    tts, finite, lu, span, stats, pp, steps_ran = serve(True)
    btts, bfinite, blu, bspan, bstats, bpp, _ = serve(False)
    done = len(tts)
    # One case at a time, the comparators, on the same work as the server's: a sample
    # of the stream's cases of each model spanning its grid sizes (every k-th case in the
    # order of N), each stepped alone for a fraction of its steps; the stream's time is
    # the sum over all its cases of the per-cell-update time of the sample case of the
    # same model nearest in N, times the case's cell updates in the server (a case the
    # server stopped early -- diverged -- counts with the steps it ran there).
    ran = dict(zip([id(c) for c in stream], steps_ran))

    def strata(cases, m):
        by_n = sorted(cases, key=lambda c: c['n'])
        kk = max(1, len(by_n) // max(1, m))
        return by_n[kk // 2::kk][:m]
    pp_cases = [c for c in stream if c['model'] == 'PP16']
    samples = {'AC': strata(ac, args.serving_sample), 'PP16': strata(pp_cases, max(1, args.serving_sample // 2))}

    one_stream = torch.cuda.Stream()

    def one_at_a_time(precision):
        rates, out = {}, {}
        for model, sample in samples.items():
            rates[model] = []
            for c in sample:
                gc = capi.GpuCase(serving_case(c, precision), c['n'], c['n'], False)
                gc.init(c['init'], c['params'])
                gc.step(2, one_stream.cuda_stream)
                torch.cuda.synchronize()
                nst = max(20, min(1000, c['steps']) // args.serving_fraction)
                ta = time.perf_counter()
                gc.step(nst, one_stream.cuda_stream)  # a caller's stream, as the server's lanes
                gc.get('rho')
                el = time.perf_counter() - ta
                rates[model].append((c['n'], el / (c['n'] * c['n'] * nst)))  # seconds per cell update
                del gc
        total = 0.0
        for c in stream:
            r = rates[c['model']]
            ns = np.array([x[0] for x in r])
            total += r[int(np.argmin(np.abs(ns - c['n'])))][1] * c['n'] * c['n'] * ran[id(c)]
        for model, r in rates.items():
            out[model] = {'sample_cases': len(r), 'sample_n': [int(x[0]) for x in r],
                          'mlups_sample_median': round(float(np.median([1e-6 / x[1] for x in r])), 2)}
        out['steps_timed_per_case'] = f'max(20, min(1000, steps) / {args.serving_fraction})'
        out['stream_seconds_projected'] = round(total, 3)
        out['stream_cases_per_s_projected'] = round(len(stream) / total, 4)
        return out

    fp64 = one_at_a_time('fp64')
    fp32 = one_at_a_time('fp32dev')
    cps = done / span if span > 0 else 0.0
    bcps = len(btts) / bspan if bspan > 0 else 0.0
    # all cases of the stream (Allen-Cahn and D2V16) per second: the server against one
    # case at a time on the same work
    all_cps, ball_cps = len(stream) / span, len(stream) / bspan
    return {
        'workload': f'{args.serving_cases}-case seeded stream (Poisson 20/s, N lognormal median 256 in '
                    f'[64,1024], {args.serving_steps} steps each, FP32 storage): {len(ac)} Allen-Cahn droplets/'
                    f'bubbles (R=N/5, density ratio U[2,100], sigma U[1e-4,1e-2]) and {len(stream) - len(ac)} '
                    f'D2V16 pseudopotential cases (T/Tc U[0.6,0.85], CS a=0.5 b=4, rho_c(1+0.01U) noise, '
                    f'lattice speed {D2V16_C}, Mu0 {PP_MU0}); checked every 1000 steps',
        'allen_cahn': 'completed, span, cases_per_s, mlups and tts are of the Allen-Cahn cases',
        'completed': done, 'finite': finite, 'span_s': round(span, 3), 'cases_per_s': round(cps, 4),
        'mlups': round(lu / span / 1e6, 2) if span > 0 else None,
        'mlups_all_cases': round(stats.cell_updates / span / 1e6, 2) if span > 0 else None,
        'tts_p50_s': round(float(np.percentile(tts, 50)), 4) if tts else None,
        'tts_p99_s': round(float(np.percentile(tts, 99)), 4) if tts else None,
        'pseudopotential_d2v16': pp,
        'max_resident': stats.max_resident, 'graphs_captured': stats.graphs_captured, 'chunks': stats.chunks,
        'bytes_peak': stats.bytes_peak, 'max_bytes': stats.max_bytes, 'solo_steps': stats.solo_steps,
        'burst': {'how': 'the same cases all submitted at once (capacity)', 'completed': len(btts),
                  'finite': bfinite, 'span_s': round(bspan, 3),
                  'cases_per_s': round(bcps, 4) if bspan > 0 else None,
                  'mlups': round(blu / bspan / 1e6, 2) if bspan > 0 else None,
                  'mlups_all_cases': round(bstats.cell_updates / bspan / 1e6, 2) if bspan > 0 else None,
                  'tts_p50_s': round(float(np.percentile(btts, 50)), 4) if btts else None,
                  'tts_p99_s': round(float(np.percentile(btts, 99)), 4) if btts else None,
                  'pseudopotential_d2v16': bpp,
                  'max_resident': bstats.max_resident, 'bytes_peak': bstats.bytes_peak},
        'one_at_a_time_fp64': fp64, 'one_at_a_time_fp32': fp32,
        # the gain of the server over one case at a time: against the plain FP64 path
        # (precision and batching together) and against FP32 storage without batching
        # (batching alone), paced at the stream's arrivals and at capacity
        'stream_cases_per_s': round(all_cps, 4), 'capacity_stream_cases_per_s': round(ball_cps, 4),
        'vs_one_at_a_time_fp64': round(all_cps / fp64['stream_cases_per_s_projected'], 2),
        'vs_one_at_a_time_fp32': round(all_cps / fp32['stream_cases_per_s_projected'], 2),
        'capacity_vs_one_at_a_time_fp64': round(ball_cps / fp64['stream_cases_per_s_projected'], 2),
        'capacity_vs_one_at_a_time_fp32': round(ball_cps / fp32['stream_cases_per_s_projected'], 2),
    }


# ---------------------------------------------------------------- pseudopotential D2V16

def cs_pressure(rho, T, a=PP_A):
    """Carnahan-Starling pressure of Ark/Lib/nonidealEoS.h (R = 1, b = 4: eta = rho)."""
    return rho * T * (1 + rho + rho ** 2 - rho ** 3) / (1 - rho) ** 3 - a * rho ** 2


def maxwell_densities(Tr: float) -> tuple[float, float]:
    """Coexisting vapour and liquid densities of the Carnahan-Starling EOS at T = Tr Tc by
    the Maxwell construction: the saturation pressure p_s at which the two branches
    enclose equal areas, int_{rho_v}^{rho_l} (p - p_s) / rho^2 drho = 0 (equal areas in
    the specific volume 1/rho); p_s by bisection, the area being monotone in p_s."""
    import numpy as np
    from scipy.integrate import quad
    from scipy.optimize import brentq
    T = Tr * PP_TC
    grid = np.linspace(1e-5, 0.7, 70001)
    pr = cs_pressure(grid, T)
    d = np.diff(pr)
    i1 = int(np.argmax(d < 0))                  # the vapour-side spinodal (local maximum)
    i2 = i1 + int(np.argmax(d[i1:] > 0))        # the liquid-side spinodal (local minimum)
    s1, s2 = grid[i1], grid[i2]

    def branches(ps):
        return (brentq(lambda r: cs_pressure(r, T) - ps, 1e-12, s1, xtol=1e-15),
                brentq(lambda r: cs_pressure(r, T) - ps, s2, 0.999, xtol=1e-15))

    def area(ps):
        rv, rl = branches(ps)
        return quad(lambda r: (cs_pressure(r, T) - ps) / r ** 2, rv, rl, limit=200, epsabs=1e-14)[0]
    lo, hi = max(cs_pressure(s2, T), 1e-14), cs_pressure(s1, T)
    for _ in range(100):
        mid = 0.5 * (lo + hi)
        if area(mid) > 0:
            lo = mid
        else:
            hi = mid
    rv, rl = branches(0.5 * (lo + hi))
    return float(rv), float(rl)


C3 = dict(n=1024, Tr=0.7, steps=50000)


def c3_case(precision: str):
    from mpdugks_gb300 import capi
    return capi.make_case('PP16', precision, Tr=C3['Tr'], aCS=PP_A, Tc_CS=PP_TC, d2v16_c=D2V16_C, Mu0=PP_MU0)


def phase_densities(rho) -> dict:
    """Vapour and liquid densities of a separated field: the mean density of the cells
    below / above the critical density, and the 1st / 99th percentiles."""
    import numpy as np
    r = rho.ravel()
    lo, hi = r[r < PP_RHO_C], r[r >= PP_RHO_C]
    return {'vapour_mean': float(lo.mean()) if lo.size else None, 'liquid_mean': float(hi.mean()) if hi.size else None,
            'p1': float(np.percentile(r, 1)), 'p99': float(np.percentile(r, 99)),
            'liquid_fraction': float(hi.size / r.size)}


def pseudopotential_bench(steps: int = 100) -> dict:
    """The pseudopotential configuration (C3): D2V16, 1024x1024 periodic, Carnahan-Starling
    a = 0.5, b = 4, R = 1 at T = 0.7 Tc, density rho_c (1 + 0.01 U(-1, 1)) from seed; FP32
    storage against the plain FP64 path on the same grid: MLUPS, HBM fraction and the
    per-field errors after `steps` steps, beside the FMA-contracted FP64 variant against
    plain FP64 (spinodal growth amplifies any difference, rounding included)."""
    import torch
    n = C3['n']
    st = torch.cuda.Stream()
    out, cases = {}, {}
    for arm in ('fp32dev', 'fp32dev_single_pass', 'fp64', 'fp64fma'):
        from mpdugks_gb300 import capi
        prec = 'fp32dev' if arm.startswith('fp32') else arm
        # the FP32 handle takes the three-pass step; the single-pass form beside it
        if arm == 'fp32dev_single_pass':
            os.environ['DUGKS_PP_PASSES'] = '1'
        g = capi.GpuCase(c3_case(prec), n, n, False)
        os.environ.pop('DUGKS_PP_PASSES', None)
        g.init('pp_noise', [PP_RHO_C, 0.01], seed=2026)
        g.step(3, st.cuda_stream)
        ms, launches, _ = timed_steps(g, steps, st)
        mlups = n * n * steps / (ms * 1e-3) / 1e6
        # compulsory bytes per cell-update: 16 distributions (+ the 2-component force)
        # read and written, 4 B each in FP32 storage, 8 B in FP64
        algo = 144 if prec == 'fp32dev' else 288
        out[arm] = {'mlups': round(mlups, 2), 'ms_per_step': round(ms / steps, 4), 'launches': launches,
                    'algorithmic_bytes_per_cell': algo, 'achieved_gbs': round(mlups * algo / 1e3, 1),
                    'hbm_frac': round(mlups * algo / 1e3 / load_peaks()[0], 4), 'peak': load_peaks()[1]}
        if arm == 'fp32dev_single_pass':
            # what the single-pass step stores per cell-update: 16 FP32 remainders, the FP64
            # density and velocity, the psi pair and sign, 4 face-force planes, read and
            # written; the pressure and the cell force written
            out[arm]['stored_bytes_per_cell'] = 248
        cases[arm] = g
    errs = field_errors(cases['fp32dev'], cases['fp64'])
    efma = field_errors(cases['fp64fma'], cases['fp64'])
    for e in (errs, efma):
        del e['phi']
    return {
        'workload': f'D2V16 pseudopotential (C3), {n}x{n} periodic, Carnahan-Starling a=0.5 b=4 R=1, '
                    f'T = {C3["Tr"]} Tc, rho_c(1 + 0.01 U(-1,1)) seeded, lattice speed {D2V16_C}, Mu0 {PP_MU0}',
        'fp32': out['fp32dev'], 'fp32_single_pass': out['fp32dev_single_pass'], 'fp64': out['fp64'],
        'fp64fma': out['fp64fma'],
        'fp32_speedup': round(out['fp32dev']['mlups'] / out['fp64']['mlups'], 2),
        'single_pass_vs_three_pass': round(out['fp32dev_single_pass']['mlups'] / out['fp32dev']['mlups'], 3),
        'fp32_error_vs_fp64': {'steps': steps + 3, 'fields': errs},
        'fp64fma_error_vs_fp64': {'steps': steps + 3, 'fields': efma},
        'maxwell_densities': maxwell_densities(C3['Tr']),
    }


def c3_full(args) -> dict:
    """C3 to its full step count: density range, phase densities against the Maxwell
    construction, mass drift and finiteness every 5000 steps, MLUPS."""
    import torch
    from mpdugks_gb300 import capi
    n, total = C3['n'], args.full_steps or C3['steps']
    prec = args.precision or 'fp32dev'
    st = torch.cuda.Stream()
    g = capi.GpuCase(c3_case(prec), n, n, False)
    g.init('pp_noise', [PP_RHO_C, 0.01], seed=2026)
    m0 = g.reduce().sum_rho
    rows, ms_total, done = [], 0.0, 0
    while done < total:
        k = min(5000, total - done)
        ms, _, _ = timed_steps(g, k, st)
        ms_total += ms
        done += k
        rho = g.get('rho')
        import numpy as np
        fin = bool(np.isfinite(rho).all())
        row = {'steps': done, 'ms_per_step': round(ms / k, 4), 'finite': fin,
               'mass_rel_drift': (float(rho.sum()) - m0) / m0, 'max_abs_u': float(np.max(np.abs(g.get('u'))))}
        row.update(phase_densities(rho))
        rows.append(row)
        if not fin:
            break
    return {'workload': 'C3 D2V16 pseudopotential coexistence 1024x1024', 'precision': prec, 'steps': done,
            'mlups': round(n * n * done / (ms_total * 1e-3) / 1e6, 2), 'maxwell_densities': maxwell_densities(C3['Tr']),
            'history': rows}


# ---------------------------------------------------------------- scheme variants

def scheme_variants_bench(steps: int = 20, precision: str = 'fp64') -> dict:
    """The reference's alternative face reconstruction (UW) and wall treatment (NEE)
    beside the defaults (CD, bounce-back) on the same grid, in one precision (the plain
    FP64 path or FP32 storage): a 1024x1024 periodic HCZ droplet (CD / UW) and the
    512x2048 Rayleigh-Taylor box with walls (BB / NEE); MLUPS over `steps` steps after 3
    warm-up steps."""
    import torch
    from mpdugks_gb300 import capi
    st = torch.cuda.Stream()
    out = {}
    drop = dict(Mu0=0.02, M_Phi=0.02, W=4.0, Sigma=1e-3, RhoL=10.0, RhoV=1.0)
    rt = WORKLOADS['rt512x2048']
    runs = [('cd', 'HCZ', drop, 1024, 1024, False, 'ac_drop_inside', [200.0], {}),
            ('uw', 'HCZ', drop, 1024, 1024, False, 'ac_drop_inside', [200.0], dict(scheme='UW')),
            ('bb', 'HCZ', case_kw(rt), rt['nx'], rt['ny'], True, 'ac_rt', rt['init'], {}),
            ('nee', 'HCZ', case_kw(rt), rt['nx'], rt['ny'], True, 'ac_rt', rt['init'], dict(wall='NEE'))]
    for tag, model, kw, nx, ny, walls, init, params, extra in runs:
        g = capi.GpuCase(capi.make_case(model, precision, **kw, **extra), nx, ny, walls)
        g.init(init, params)
        g.step(3, st.cuda_stream)
        ms, launches, _ = timed_steps(g, steps, st)
        out[tag] = {'grid': f'{nx}x{ny}', 'mlups': round(nx * ny * steps / (ms * 1e-3) / 1e6, 2),
                    'ms_per_step': round(ms / steps, 4), 'launches_per_step': launches // steps}
        del g
    return {'precision': 'fp64 (reference-exact rounding)' if precision == 'fp64' else precision, 'steps': steps,
            'droplet_1024x1024': {'cd': out['cd'], 'uw': out['uw']},
            'rayleigh_taylor_512x2048': {'bounce_back': out['bb'], 'nee': out['nee']}}


# ---------------------------------------------------------------- GPU arms

def field_errors(a, b):
    """Per-field max-norm and L2 error of case a against case b, relative to b (linf, l2),
    and the max-norm difference in lattice units (linf_abs) beside the field's max-norm
    (max_abs): a velocity that starts from rest is tiny after a few steps, and its
    relative error says little on its own."""
    import numpy as np
    out = {}
    for k in ('rho', 'u', 'v', 'p', 'phi'):
        x, y = a.get(k), b.get(k)
        d = x - y
        ny = float(np.max(np.abs(y)))
        dmax = float(np.max(np.abs(d)))
        out[k] = {'linf': dmax / ny if ny else dmax,
                  'l2': float(np.linalg.norm(d) / np.linalg.norm(y)) if ny else 0.0,
                  'linf_abs': dmax, 'max_abs': ny}
    return out


def developed_flow_errors(steps: int = 300) -> dict:
    """FP32 against FP64 on the 512x2048 Rayleigh-Taylor case after `steps` steps, beside
    the FMA-contracted FP64 variant against the same FP64 run: the instability
    amplifies any difference (rounding included), so the FMA column shows the
    amplification the FP32 column shares."""
    from mpdugks_gb300 import capi
    wl = WORKLOADS['rt512x2048']
    kw = case_kw(wl)
    runs = {}
    for prec in ('fp32dev', 'fp64', 'fp64fma'):
        g = capi.GpuCase(capi.make_case('HCZ', prec, **kw), wl['nx'], wl['ny'], True)
        g.init('ac_rt', wl['init'])
        g.step(steps)
        runs[prec] = g
    return {'workload': wl['name'], 'steps': steps,
            'fp32_vs_fp64': field_errors(runs['fp32dev'], runs['fp64']),
            'fp64fma_vs_fp64': field_errors(runs['fp64fma'], runs['fp64'])}


def rt_fronts(phi, nx: int, yc: float) -> dict:
    """Rayleigh-Taylor fronts of a phi field [ny][nx] (heavy phase phi = 1 above the
    interface): spike tip = lowest row with phi > 1/2 somewhere, bubble tip = highest row
    with phi < 1/2 somewhere, both relative to the initial mean height yc*L in units of
    L = nx; mixing zone = rows whose x-mean of phi lies in (0.01, 0.99), in units of L."""
    import numpy as np
    heavy = np.nonzero((phi > 0.5).any(axis=1))[0]
    light = np.nonzero((phi < 0.5).any(axis=1))[0]
    mean = phi.mean(axis=1)
    mix = np.nonzero((mean > 0.01) & (mean < 0.99))[0]
    c = yc * nx
    return {'spike': round((float(heavy.min()) + 0.5 - c) / nx, 5) if heavy.size else None,
            'bubble': round((float(light.max()) + 0.5 - c) / nx, 5) if light.size else None,
            'mixing_zone': round(float(mix.size) / nx, 5)}


def slabs_bench(args, wl, nparts: int) -> dict:
    """The workload split along y into `nparts` slab partitions on this GPU (dugks_slabs_*,
    halo rows exchanged by device copies after every step), against the undivided case:
    the cost of the decomposition's exchange and of the partitions' smaller launches.
    Host wall time around `steps` steps followed by a synchronising reduction (the
    partitions run on the library's own stream)."""
    import time
    from mpdugks_gb300 import capi
    nx, ny = wl['nx'], wl['ny']
    cells = nx * ny
    steps = max(10, args.steps // 10)
    out = {'workload': wl['name'], 'partitions': nparts, 'steps': steps, 'precision': 'fp32dev'}
    for label, n in (('undivided', 0), ('slabs', nparts)):
        if n:
            run = capi.Slabs(capi.make_case('HCZ', 'fp32dev', **case_kw(wl)), nx, ny, True, n)
        else:
            run = capi.GpuCase(capi.make_case('HCZ', 'fp32dev', **case_kw(wl)), nx, ny, True)
        run.init('ac_rt', wl['init'])
        run.step(args.warmup)
        run.reduce()
        t0 = time.perf_counter()
        run.step(steps)
        r = run.reduce()
        dt = time.perf_counter() - t0
        out[label] = {'mlups': round(cells * steps / dt / 1e6, 1), 'ms_per_step': round(dt * 1e3 / steps, 4),
                      'sum_rho': r.sum_rho}
        run.close()
    out['slabs_vs_undivided'] = round(out['slabs']['mlups'] / out['undivided']['mlups'], 4)
    return out


def full_run(args, wl) -> dict:
    """The configuration run to its full step count: time per 1000 steps (CUDA events),
    mass and phase-field drift, density residual, finiteness and the fronts of the
    instability every 1000 steps."""
    import torch
    from mpdugks_gb300 import capi
    prec = args.precision or wl['precision']
    nx, ny, n = wl['nx'], wl['ny'], args.full_steps or wl['full_steps']
    kw = case_kw(wl)
    stream = torch.cuda.Stream()
    gc = capi.GpuCase(capi.make_case('HCZ', prec, **kw), nx, ny, True)
    gc.init('ac_rt', wl['init'])
    r0 = gc.reduce()
    T = (nx / (kw['Gy'] * 0.5)) ** 0.5  # T = sqrt(L / (g At)), At = 0.5
    dt = 0.5                            # CFL dx / max|xi| of the reference (Ark/Constant/ZeroNamespace.h)
    rows, total_ms, done = [], 0.0, 0
    while done < n:
        k = min(1000, n - done)
        ms, _, _ = timed_steps(gc, k, stream)
        total_ms += ms
        done += k
        r = gc.reduce()
        fin = gc.check_finite() == 0
        row = {'steps': done, 't_over_T': round(done * dt / T, 4), 'ms_per_step': round(ms / k, 4),
               'sum_rho_rel_drift': (r.sum_rho - r0.sum_rho) / r0.sum_rho,
               'sum_phi_rel_drift': (r.sum_phi - r0.sum_phi) / r0.sum_phi,
               'residual': r.residual, 'finite': fin}
        row.update(rt_fronts(gc.get('phi').reshape(ny, nx), nx, wl['yc']))
        rows.append(row)
        if not fin:
            break
    cells = nx * ny
    return {'workload': wl['name'], 'precision': prec, 'steps': done, 'seconds': round(total_ms / 1e3, 3),
            'mlups': round(cells * done / (total_ms * 1e-3) / 1e6, 3), 'T_steps': round(T / dt, 1),
            'history': rows}


def timed_steps(gc, n: int, stream, clocks_idx=None):
    """n steps on `stream` bracketed by CUDA events on that stream; (ms, launches, clocks)."""
    import torch
    torch.cuda.synchronize()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    sampler = ClockSampler(clocks_idx) if clocks_idx is not None else None
    if sampler:
        sampler.__enter__()
    l0 = gc.launches
    ev0.record(stream)
    gc.step(n, stream.cuda_stream)
    ev1.record(stream)
    torch.cuda.synchronize()
    launches = gc.launches - l0
    if sampler:
        sampler.__exit__(None, None, None)
    return ev0.elapsed_time(ev1), launches, (sampler.summary() if sampler else None)


def run_ours(args, wl, rank, world, local):
    import numpy as np
    import torch
    import torch.distributed as dist
    from mpdugks_gb300 import capi

    torch.cuda.set_device(local)
    dev_index = torch.cuda.current_device()
    if world > 1:
        dist.init_process_group('nccl')

    def barrier():
        if world > 1:
            dist.barrier()

    def max_over_ranks(x: float) -> float:
        t = torch.tensor([x], dtype=torch.float64, device='cuda')
        if world > 1:
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t.item())

    nx, ny = wl['nx'], wl['ny']
    cells = nx * ny
    kw = case_kw(wl)
    prec = args.precision or wl['precision']
    stream = torch.cuda.Stream()

    gc = capi.GpuCase(capi.make_case('HCZ', prec, **kw), nx, ny, True)
    gc.init('ac_rt', wl['init'])
    gc.step(args.warmup, stream.cuda_stream)
    barrier()
    ms, launches, clocks = timed_steps(gc, args.steps, stream, dev_index)
    barrier()
    ms_max = max_over_ranks(ms)
    mlups_total = world * cells * args.steps / (ms_max * 1e-3) / 1e6
    finite = gc.check_finite() == 0
    red = gc.reduce()

    hbm_peak, peak_kind = load_peaks()
    step_ms = ms / args.steps
    algo = ALGO_BYTES[prec]
    achieved = algo * cells / (step_ms * 1e-3) / 1e9
    if prec == 'fp32dev':
        kernel = 'k_stream32 (the fused step: one launch per step)'
        phase = None
    else:
        nprof = max(10, min(100, args.steps))
        ph = gc.step_profiled(nprof, stream.cuda_stream)
        phase = [round(p / nprof, 5) for p in ph]
        kernel = 'one DUGKS step (k_collide + k_faces_ac + k_update)'
    traffic = TRAFFIC_BYTES.get(prec)
    roofline = {'bound': 'hbm', 'achieved': round(achieved, 2), 'peak': hbm_peak, 'unit': 'GB/s',
                'frac': round(achieved / hbm_peak, 5),
                'traffic': None if traffic is None else int(traffic * cells),
                'traffic_source': None if traffic is None else 'ncu DRAM bytes of one launch at 3072x3072, '
                                                               'scaled by the cell count',
                'kernel': kernel, 'algorithmic_bytes_per_cell': algo,
                'stored_bytes_per_cell': STORED_BYTES[prec],
                'stored_gbs': round(STORED_BYTES[prec] * cells / (step_ms * 1e-3) / 1e9, 2),
                'cells_per_launch': cells, 'peak_source': f'{peak_kind} hbm_gbs (copy bandwidth)'}
    if phase:
        roofline['phase_ms'] = phase
        roofline['note'] = 'FP64 path: bound by the FP64 pipe, not HBM (fp64_pipe)'
        roofline['fp64_pipe'] = fp64_pipe(cells * args.steps / (ms * 1e-3))

    # ---- the plain FP64 path on the same grid, and the FP32-vs-FP64 field errors
    fp64 = None
    gx = None
    if prec == 'fp32dev' and not args.no_fp64:
        g64 = capi.GpuCase(capi.make_case('HCZ', 'fp64', **kw), nx, ny, True)
        g64.init('ac_rt', wl['init'])
        g64.step(3, stream.cuda_stream)
        k64 = args.fp64_steps
        ms64, _, _ = timed_steps(g64, k64, stream)
        n_cmp = 3 + k64
        g32 = capi.GpuCase(capi.make_case('HCZ', 'fp32dev', **kw), nx, ny, True)
        g32.init('ac_rt', wl['init'])
        g32.step(n_cmp, stream.cuda_stream)
        torch.cuda.synchronize()
        errs = field_errors(g32, g64)
        del g32
        m64 = cells * k64 / (ms64 * 1e-3) / 1e6
        fp64 = {'value': round(m64, 3), 'unit': 'MLUPS', 'steps': k64, 'ms_per_step': round(ms64 / k64, 4),
                'precision': 'fp64 (reference-exact rounding)',
                'fp32_speedup': round(mlups_total / world / m64, 2),
                'fp32_error_vs_fp64': {'steps': n_cmp, 'fields': errs},
                'fp64_pipe': fp64_pipe(cells * k64 / (ms64 * 1e-3)),
                'developed_flow': developed_flow_errors()}
        gx = g64
    # ---- end to end through the C ABI with host buffers: upload the FP64 initial
    # state (the reference's CellArray contents) from pinned host memory, K steps,
    # reductions, and the five macroscopic fields back to pinned host memory
    src = gx
    if src is None:
        src = capi.GpuCase(capi.make_case('HCZ', 'fp64', **kw), nx, ny, True)
    src.init('ac_rt', wl['init'])
    pf = torch.empty((9, ny, nx), dtype=torch.float64).pin_memory()
    ph_ = torch.empty((9, ny, nx), dtype=torch.float64).pin_memory()
    pa = torch.empty((len(capi.FIELDS), ny, nx), dtype=torch.float64).pin_memory()
    src._check(src.lib.dugks_gpu_get_dist(src.h, 0, pf.data_ptr()))
    src._check(src.lib.dugks_gpu_get_dist(src.h, 1, ph_.data_ptr()))
    for k in range(len(capi.FIELDS)):
        src._check(src.lib.dugks_gpu_get_field(src.h, k, C.c_void_p(pa[k].data_ptr())))
    del src, gx
    outs = [torch.empty((ny, nx), dtype=torch.float64).pin_memory() for _ in range(5)]
    barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    gc._check(gc.lib.dugks_gpu_upload(gc.h, pf.data_ptr(), ph_.data_ptr(), pa.data_ptr()))
    gc.step(args.steps, stream.cuda_stream)
    r2 = gc.reduce()
    gc._check(gc.lib.dugks_gpu_download(gc.h, *[o.data_ptr() for o in outs]))
    torch.cuda.synchronize()
    e2e_s = max_over_ranks(time.perf_counter() - t0)
    e2e_mlups = world * cells * args.steps / e2e_s / 1e6
    h2d = (pf.numel() + ph_.numel() + pa.numel()) * 8 / args.steps
    d2h = (5 * cells * 8 + 32) / args.steps

    serving = None
    if rank == 0 and not args.no_serving:
        serving = serving_bench(args)
    pseudo = None
    if rank == 0 and not args.no_pseudopotential:
        pseudo = pseudopotential_bench(args.pp_steps)
    variants = variants32 = None
    if rank == 0 and not args.no_fp64:  # the scheme variants in FP64 and in FP32 storage
        variants = scheme_variants_bench()
        variants32 = scheme_variants_bench(precision='fp32dev')

    if rank == 0:
        cpu = None
        if not args.no_cpu_baseline:
            cpu, _, _ = cpu_baseline(wl, args.cpu_seconds, args.cpu_steps)
        line = {
            'metric': 'MLUPS', 'value': round(mlups_total, 3), 'unit': 'MLUPS', 'n_gpus': world,
            'steps': args.steps, 'warmup': args.warmup, 'ms_per_step': round(ms_max / args.steps, 5),
            'higher_is_better': True, 'scaling': 'weak', 'vs_baseline': None,
            'dtype': 'f32 storage and arithmetic (the phase field a float-float pair), f64 domain sums' if prec == 'fp32dev' else 'f64',
            'data': 'synthetic (seeded Rayleigh-Taylor initial condition, no dataset)',
            'config': {'workload': wl['name'], 'cells': cells, 'precision': prec,
                       'l2_flush': 'none needed: the state read and written each step is larger than the 129 MB L2',
                       'parallelism': f'{world} independent replicas' if world > 1 else 'single GPU'},
            'roofline': roofline,
            'fp64_same_grid': fp64,
            'cpu_baseline': cpu,
            'e2e': {'value': round(e2e_mlups, 3), 'unit': 'MLUPS', 'h2d_bytes_per_step': int(h2d),
                    'd2h_bytes_per_step': int(d2h),
                    'how': 'C ABI with pinned host buffers (the upload read in place by the library\'s '
                           'conversion kernels over NVLink-C2C): upload the FP64 initial state, K steps, '
                           'reductions, download 5 fields'},
            'serving': serving,
            'pseudopotential_d2v16': pseudo,
            'fp64_scheme_variants': variants,
            'fp32_scheme_variants': variants32,
            'gpu_launches': int(launches),
            'clocks': clocks,
            'state_finite': finite,
            'sum_rho': red.sum_rho,
            'sum_rho_e2e': r2.sum_rho,
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument('--gpus', type=int, default=1)
    ap.add_argument('--steps', type=int, default=1000)
    ap.add_argument('--warmup', type=int, default=20)
    ap.add_argument('--impl', default='ours', choices=['ours', 'reference'])
    ap.add_argument('--workload', default='rt8192', choices=sorted(WORKLOADS))
    ap.add_argument('--precision', default=None, choices=['fp32dev', 'fp64', 'fp64fma'],
                    help='default: fp32dev for rt8192, fp64 (reference-exact rounding) for rt512x2048')
    ap.add_argument('--fp64-steps', type=int, default=10, help='timed steps of the FP64 arm on the same grid')
    ap.add_argument('--no-fp64', action='store_true', help='skip the FP64 arm on the same grid')
    ap.add_argument('--cpu-steps', type=int, default=0, help='CPU baseline steps (0: about --cpu-seconds)')
    ap.add_argument('--cpu-seconds', type=float, default=15.0)
    ap.add_argument('--no-cpu-baseline', action='store_true')
    ap.add_argument('--no-serving', action='store_true', help='skip the serving-stream measurement')
    ap.add_argument('--no-pseudopotential', action='store_true', help='skip the D2V16 FP32/FP64 measurement')
    ap.add_argument('--serving-only', action='store_true', help='run only the serving-stream measurement')
    ap.add_argument('--pseudopotential-only', action='store_true',
                    help='run only the D2V16 FP32/FP64 measurement (--pp-steps timed steps)')
    ap.add_argument('--pp-steps', type=int, default=100)
    ap.add_argument('--c3-full', action='store_true',
                    help='run the D2V16 coexistence configuration (C3) to its 50000 steps (--precision, --full-steps)')
    ap.add_argument('--serving-cases', type=int, default=SERVING['cases'])
    ap.add_argument('--serving-steps', type=int, default=SERVING['steps'])
    ap.add_argument('--serving-sample', type=int, default=24,
                    help='Allen-Cahn cases (spanning the grid sizes) solved one at a time for comparison')
    ap.add_argument('--serving-fraction', type=int, default=10,
                    help='the one-at-a-time comparators time 1/fraction of each sample case\'s steps')
    ap.add_argument('--profile-steps', type=int, default=0,
                    help='only run this many steps of the workload (for ncu) and exit')
    ap.add_argument('--grid', default=None, help='NXxNY override of the grid (profiling runs only)')
    ap.add_argument('--full-run', action='store_true',
                    help='run the workload for its configured step count (10000 at 8192^2, 20000 at 512x2048) '
                         'and print its history (timing, conservation, residual, instability fronts)')
    ap.add_argument('--full-steps', type=int, default=0, help='step count of --full-run (0: the configured one)')
    ap.add_argument('--slabs', type=int, default=0,
                    help='run only the slab decomposition of the workload into this many partitions on this GPU '
                         'against the undivided case (steps / 10 timed steps)')
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    wl = dict(WORKLOADS[args.workload])
    rank, world, local = env_dist()
    if args.profile_steps:
        # a short plain run of the workload for profilers (ncu); no timing, no JSON line
        from mpdugks_gb300 import capi
        if args.grid:
            wl['nx'], wl['ny'] = (int(x) for x in args.grid.lower().split('x'))
        prec = args.precision or wl['precision']
        gc = capi.GpuCase(capi.make_case('HCZ', prec, **case_kw(wl)), wl['nx'], wl['ny'], True)
        gc.init('ac_rt', wl['init'])
        gc.step(args.profile_steps)
        r = gc.reduce()
        print(f'profile run: {wl["nx"]}x{wl["ny"]}, {args.profile_steps} steps, precision {prec}, '
              f'sum rho {r.sum_rho!r}')
        return 0
    if args.grid:
        ap.error('--grid is for --profile-steps runs only')
    if args.impl == 'reference':
        return run_reference(args, wl, rank, world)
    if args.full_run:
        import torch
        torch.cuda.set_device(local)
        print(json.dumps({'full_run': full_run(args, wl)}), flush=True)
        return 0
    if args.serving_only:
        import torch
        torch.cuda.set_device(local)
        print(json.dumps({'serving': serving_bench(args)}), flush=True)
        return 0
    if args.slabs:
        import torch
        torch.cuda.set_device(local)
        print(json.dumps({'slabs': slabs_bench(args, wl, args.slabs)}), flush=True)
        return 0
    if args.c3_full:
        import torch
        torch.cuda.set_device(local)
        print(json.dumps({'c3_full': c3_full(args)}), flush=True)
        return 0
    if args.pseudopotential_only:
        import torch
        torch.cuda.set_device(local)
        print(json.dumps({'pseudopotential_d2v16': pseudopotential_bench(args.pp_steps)}), flush=True)
        return 0
    return run_ours(args, wl, rank, world, local)


if __name__ == '__main__':
    sys.exit(main())
