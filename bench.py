#!/usr/bin/env python3
"""Benchmark of the batch-SOM hot path on GB300: one step = one SOM_Batch training epoch.

Workload (default, the shape of the >=10x target): square 64x64 map, D=16 float32 features, N=12,582,912 samples (the
HEALPix nside=1024 pixel count) from the seeded correlated log-normal generator (decontamination_gb300.synthetic,
seed 2), weights U[-1, 1], sigma0 = 32 with the reference's 1/(1+2e/E) decay over a 20-epoch schedule.

  value     epochs with the catalogue resident in HBM (805 MB > L2, so no flush is needed): each epoch is one fused
            BMU + error pass, the per-BMU segmented sums and the neighbourhood update, timed with CUDA events;
            metric N*M / epoch time in Gsample.unit/s.
  e2e       the same metric through the public API call a user makes, SOM_Batch.train(X, n_epochs=1) on a pinned
            host tensor: host->device copy of the catalogue, training pass, error pass and device->host copy of the
            weights, history and errors every step.
  fp32_form the plain FP32 CUDA-core form of the same epoch (the tensor-core path's baseline).
  parity    on the full catalogue after the timed epochs: the BMUs of the tensor-core pass against an independent
            evaluation (float32 GEMM distances for the three nearest units, then the reference's typing), rows whose
            two best distances are tied within float32 rounding counted and adjudicated by float64 distances; the
            trained weights of one more epoch against a float64 evaluation of the same update from the same BMUs.
  sq64      the 64x64, D = 32 configuration over 50,331,648 rows (HEALPix nside=2048), generated on the device.
  serve     BMU serving on a resident 64x64, D = 16 map: Poisson arrivals, request sizes log-uniform in [1e3, 1e7].
  cpu_baseline  the reference's CPU formulation (oracle port: per-sample scatter into every unit with float32
            atomics, then the error pass) on all host cores, on a bounded prefix of the catalogue.

`--impl reference` times only that CPU formulation (rank 0), each step a bounded prefix of the workload, and prints
its line. `--serve` prints the serving record alone. Under torchrun every rank runs an independent replica (the path is
data-parallel; this build keeps one GPU per replica and no collective) and value = units processed by all ranks / max
time.
"""

import argparse
import gc
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOADS = {
    # the speed-up target's shape: a 64x64 map with D = 16 over the 12.6 M-row catalogue
    'sq64d16': dict(name='square 64x64 SOM, D=16, N=12582912 (HEALPix nside=1024 pixel count), sigma0=32, '
                         '20-epoch schedule', m=64, n=64, d=16, N=12_582_912, topology='square', sigma0=32.0,
                    schedule=20, seed=2),
    # the plain-FP32 training configuration's shape: hexagonal 32x32, D = 16, same catalogue
    'hex32': dict(name='hex 32x32 SOM, D=16, N=12582912 (HEALPix nside=1024 pixel count), sigma0=16, 20-epoch schedule',
                  m=32, n=32, d=16, N=12_582_912, topology='hexagonal', sigma0=16.0, schedule=20, seed=2),
    # the split-precision configuration: square 64x64, D = 32, N = 50,331,648 (HEALPix nside 2048)
    'sq64': dict(name='square 64x64 SOM, D=32, N=50331648 (HEALPix nside=2048 pixel count), sigma0=32, '
                      '20-epoch schedule', m=64, n=64, d=32, N=50_331_648, topology='square', sigma0=32.0,
                 schedule=20, seed=3),
}
METRIC = 'SOM epoch Gsample·unit/s'
UNIT = 'Gsample·unit/s'
# DRAM traffic (bytes read + written) of one tensor-core BMU pass per catalogue row, from ncu captures of tc_pass_kernel
# on 4,194,304-row cases of each workload (summaries under profiles/). The pass streams every row once (the samples,
# the BMU, the unit operand from L2), so the traffic of a full launch scales with N.
K1_DRAM_BYTES_PER_ROW = {'sq64d16': (269.468672e6 + 15.487488e6) / 4_194_304,
                         'hex32': (268.734208e6 + 15.436032e6) / 4_194_304}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument('--gpus', type=int, default=1)
    ap.add_argument('--steps', type=int, default=20)
    ap.add_argument('--warmup', type=int, default=3)
    ap.add_argument('--impl', default='ours', choices=['ours', 'reference'])
    ap.add_argument('--algo', default='auto', choices=['auto', 'tc', 'fp32'])
    ap.add_argument('--workload', default='sq64d16', choices=sorted(WORKLOADS))
    ap.add_argument('--n', type=int, default=None, help='catalogue rows (default: the full workload)')
    ap.add_argument('--skip-cpu', action='store_true')
    ap.add_argument('--skip-e2e', action='store_true')
    ap.add_argument('--skip-fp32', action='store_true')
    ap.add_argument('--skip-parity', action='store_true')
    ap.add_argument('--skip-sq64', action='store_true', help='no 64x64, D = 32, 50.3 M-row sub-record')
    ap.add_argument('--skip-serve', action='store_true', help='no serving sub-record')
    ap.add_argument('--skip-iter', action='store_true', help='no iteration-mode sub-record')
    ap.add_argument('--cpu-seconds', type=float, default=12.0)
    ap.add_argument('--clock-seconds', type=float, default=2.0,
                    help='the epochs also run this long after the timed ones while the clocks are sampled')
    ap.add_argument('--serve', action='store_true', help='print the BMU-serving record alone')
    ap.add_argument('--serve-seconds', type=float, default=10.0, help='arrival window of the serving run')
    ap.add_argument('--serve-rate', type=float, default=200.0, help='mean request arrivals per second')
    ap.add_argument('--serve-train', action='store_true',
                    help='mixed-training serving: a stream of training jobs of mixed grids, D and sizes')
    ap.add_argument('--jobs', type=int, default=500, help='training jobs of --serve-train')
    ap.add_argument('--train-algos', default='auto,fp32', help='distance searches compared by --serve-train')
    return ap.parse_args()


# ----------------------------------------------------------------------------------------------------------------------
# helpers
# ----------------------------------------------------------------------------------------------------------------------

class ClockSampler:
    """nvidia-smi clock / throttle-reason samples every 200 ms while active."""

    FIELDS = ('index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,'
              'clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,'
              'clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap')

    def __init__(self, gpu_id):
        self.gpu_id = gpu_id
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix='.csv')
        os.close(fd)
        cmd = ['nvidia-smi', f'--query-gpu={self.FIELDS}', '--format=csv,noheader,nounits', '-lms', '200']
        if self.gpu_id is not None:
            cmd.insert(1, f'--id={self.gpu_id}')
        try:
            self.proc = subprocess.Popen(cmd, stdout=open(self.path, 'w'), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            self.proc.wait()

    def summary(self):
        rows = []
        try:
            for line in open(self.path):
                parts = [p.strip() for p in line.split(',')]
                if len(parts) >= 9:
                    rows.append(parts)
        finally:
            os.unlink(self.path)
        if not rows:
            return {'sm_mhz': None, 'sm_max_mhz': None, 'reasons': ['unavailable'], 'samples': 0}
        sm = [float(r[1]) for r in rows if r[1].replace('.', '').isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace('.', '').isdigit()]
        names = ['hw_slowdown', 'hw_thermal_slowdown', 'sw_thermal_slowdown', 'sw_power_cap']
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == 'active'})
        loaded = [s for s in sm if mx and s > 0.5 * max(mx)] or sm
        return {'sm_mhz': statistics.median(loaded) if loaded else None, 'sm_max_mhz': max(mx) if mx else None,
                'reasons': reasons, 'samples': len(rows)}


def gpu_bus_id(torch, dev):
    try:
        p = torch.cuda.get_device_properties(dev)
        return f'{p.pci_domain_id:08X}:{p.pci_bus_id:02X}:{p.pci_device_id:02X}.0'
    except Exception:
        return None


def measured_peaks():
    try:
        with open(os.path.join(ROOT, 'MEASURED_PEAKS.json')) as f:
            return json.load(f), 'measured'
    except OSError:
        return {'hbm_gbs': 6800.0, 'bf16_tflops': 1900.0, 'bf16_tflops_sustained': 1700.0}, 'fallback'


def dist_env():
    ws = int(os.environ.get('WORLD_SIZE', '1'))
    rank = int(os.environ.get('RANK', '0'))
    local = int(os.environ.get('LOCAL_RANK', '0'))
    return ws, rank, local


def slowest_rank(t, ws, device=None):
    """The time `t` maximised over the ranks of the process group (`t` itself for one rank): the job's time is its
    slowest replica's."""
    if ws == 1:
        return float(t)
    import torch
    import torch.distributed as dist
    tt = torch.tensor([float(t)], dtype=torch.float64, device=device)
    dist.all_reduce(tt, op=dist.ReduceOp.MAX)
    return float(tt.item())


def whole_job_rate(ws, n, m, ms_per_step):
    """Gsample·unit/s of the whole job: every one of the ws ranks processes n samples against m units per step."""
    return ws * n * m / (ms_per_step * 1e-3) / 1e9


def make_data(N, w):
    from decontamination_gb300 import synthetic
    x = synthetic.correlated_lognormal(N, w['d'], w['seed'])
    w0 = synthetic.uniform_weights(w['m'] * w['n'], w['d'], w['seed'])
    return x, w0


# ----------------------------------------------------------------------------------------------------------------------
# CPU formulation of the reference (oracle port) — the reference arm and the cpu_baseline leg
# ----------------------------------------------------------------------------------------------------------------------

def cpu_epoch_rate(x, w0, w, seconds, threads=0):
    """Times one reference-formulation epoch (scatter with float32 atomics + error pass) on a prefix of x sized to
    take about `seconds`. Returns (Gsample.unit/s, prefix rows, threads, seconds measured)."""
    from oracle import somref
    M, D = w['m'] * w['n'], w['d']
    topo = somref.topography(w['m'], w['n'], w['topology'])
    nthreads = threads or os.cpu_count()

    def run(ns):
        num = np.zeros((M, D), np.float32)
        den = np.zeros(M, np.float32)
        xs = np.ascontiguousarray(x[:ns])
        rho = np.ones(ns, np.float32)
        t0 = time.perf_counter()
        somref.train_epoch_scatter(num, den, w0, topo, xs, rho, w['sigma0'], 0, w['schedule'], 'numba',
                                   threads=nthreads)
        wn = somref.OracleSOM(w['m'], w['n'], D, topology=w['topology'])._divide(num, den)
        somref.compute_errors_raw(wn, topo, xs, None, 2.0 if w['topology'] == 'square' else 1.0, 'numba',
                                  threads=nthreads)
        return time.perf_counter() - t0

    ns = 2048
    dt = run(ns)
    ns = int(min(x.shape[0], max(ns, ns * seconds / max(dt, 1e-3))))
    dt = run(ns)
    return ns * M / dt / 1e9, ns, nthreads, dt


def reference_arm(args, ws, rank):
    """The reference's CPU formulation on rank 0: each step one epoch over a prefix of the workload's catalogue; the
    line reports the measured time of those steps (the prefix rows are named in `config`)."""
    w = WORKLOADS[args.workload]
    if rank != 0:
        return
    x, w0 = make_data(min(args.n or w['N'], 400_000), w)
    M = w['m'] * w['n']
    rates, secs, rows = [], [], None
    nt = None
    t_start = time.perf_counter()
    for step in range(args.warmup + args.steps):
        r, ns, nt, dt = cpu_epoch_rate(x, w0, w, seconds=2.0)
        if step >= args.warmup:
            rates.append(r)
            secs.append(dt)
            rows = ns
    wall = time.perf_counter() - t_start
    value = statistics.median(rates)
    ms = statistics.median(secs) * 1e3
    line = {
        'impl': 'reference', 'metric': METRIC, 'value': value, 'unit': UNIT, 'n_gpus': args.gpus, 'steps': args.steps,
        'warmup': args.warmup, 'ms_per_step': ms, 'higher_is_better': True, 'scaling': 'weak', 'vs_baseline': None,
        'dtype': 'f32', 'data': 'synthetic',
        'config': {'workload': w['name'], 'rows_per_step': rows, 'units': M,
                   'formulation': 'reference CPU epoch (per-sample scatter into every unit with float32 atomics, '
                                  'then the error pass) as the oracle port in C++/OpenMP; numba, which the reference '
                                  'compiles it with, is not installed'},
        'cpu_baseline': {'value': value, 'unit': UNIT, 'cores': nt, 'kind': 'port',
                         'sample': f'first {rows} rows of the workload per step (one epoch and its error pass)'},
        'e2e': {'value': value, 'unit': UNIT, 'h2d_bytes_per_step': 0, 'd2h_bytes_per_step': 0},
        'consistency': {'steps_wall_s': wall, 'steps_x_ms_s': (args.warmup + args.steps) * ms * 1e-3},
    }
    print(json.dumps(line), flush=True)


# ----------------------------------------------------------------------------------------------------------------------
# GPU arm
# ----------------------------------------------------------------------------------------------------------------------

class EpochRunner:
    """The epoch of SOM_Batch.train with the catalogue resident on the device (same libsomgb calls)."""

    def __init__(self, torch, native, xd, w0, topo, w, algo, device):
        self.t, self.nat, self.xd, self.topo, self.w, self.dev = torch, native, xd, topo, w, device
        self.M, self.D, self.N = w['m'] * w['n'], w['d'], int(xd.shape[0])
        self.algo = native.ALGOS[algo]
        self.wcur = (torch.from_numpy(w0) if isinstance(w0, np.ndarray) else w0).to(device).contiguous()
        self.wnext = torch.empty_like(self.wcur)
        self.S = torch.empty((self.M, self.D), dtype=torch.float64, device=device)
        self.c = torch.empty(self.M, dtype=torch.float64, device=device)
        self.bmu = torch.empty(self.N, dtype=torch.int32, device=device)
        # per-feature bounds of the fixed-point sums: a property of the resident catalogue, computed once
        self.bounds = torch.zeros(self.D + 1, dtype=torch.float32, device=device)
        native.call('somgb_feature_bounds', xd.data_ptr(), None, self.N, self.D, self.bounds.data_ptr(),
                    torch.cuda.current_stream().cuda_stream)
        nbytes = native.workspace_bytes(native.OP_FIND_BMUS, self.N, self.M, self.D, self.algo)
        self.ws = torch.empty(nbytes + 256, dtype=torch.uint8, device=device)
        self.wsp = self.ws.data_ptr() + (-self.ws.data_ptr()) % 256
        self.wsb = nbytes
        # the pass's sweep-2 column-tile counter (workspace header word 2), copied on the device after every pass
        off = self.wsp - self.ws.data_ptr()
        self.sweep2_word = self.ws[off + 16:off + 24].view(torch.int64)
        self.sweep2_log = []
        self.penalty = 2.0 if w['topology'] == 'square' else 1.0
        nb = int(native.lib().somgb_neighbourhood_grid_workspace_bytes(w['m'], w['n'], self.D))
        self.upd_ws = torch.empty(nb, dtype=torch.uint8, device=device)
        # the tensor-core form regroups the catalogue's rows by BMU after each epoch (SOM_Batch.train does the same)
        self.regroup = self.algo != native.ALGO_FP32 and self.M > 256
        self.x_pass = xd     # the rows (in their order) of the last pass, which self.bmu refers to
        if self.regroup:     # two buffers of its own: the caller's catalogue is never written
            self.bufs = [torch.empty_like(xd), torch.empty_like(xd)]
            self.sort_ws = torch.empty(int(native.lib().somgb_sort_rows_workspace_bytes(self.M)), dtype=torch.uint8,
                                       device=device)
        self.epoch = 0

    def sigma(self):
        e = self.epoch % self.w['schedule']
        return max(float(np.float32(self.w['sigma0'])) / (1.0 + 2.0 * e / self.w['schedule']), 1e-12)

    def step(self, err_slot, timer=None, phases=None):
        t, nat = self.t, self.nat
        s = t.cuda.current_stream().cuda_stream
        if phases is not None:
            phases[0].record()
        self.S.zero_()
        self.c.zero_()
        if timer is not None:
            nat.call('somgb_set_kernel_timer', timer[0].cuda_event, timer[1].cuda_event)
        nat.call('somgb_train_bmu_pass', self.xd.data_ptr(), None, self.N, self.D, self.wcur.data_ptr(),
                 self.topo.data_ptr(), self.M, self.penalty, self.algo, self.bmu.data_ptr(), err_slot.data_ptr(),
                 self.wsp, self.wsb, s)
        if timer is not None:
            nat.call('somgb_set_kernel_timer', None, None)
        self.sweep2_log.append(self.sweep2_word.clone())
        if phases is not None:
            phases[1].record()
        nat.call('somgb_accumulate', self.xd.data_ptr(), None, self.bmu.data_ptr(), self.N, self.D, self.M,
                 self.bounds.data_ptr(), self.S.data_ptr(), self.c.data_ptr(), s)
        if phases is not None:
            phases[2].record()
        self.x_pass = self.xd
        if self.regroup:
            xs = self.bufs[0] if self.bufs[0] is not self.xd else self.bufs[1]
            nat.call('somgb_sort_rows', self.xd.data_ptr(), None, self.bmu.data_ptr(), self.N, self.D, self.M,
                     xs.data_ptr(), None, self.sort_ws.data_ptr(), self.sort_ws.numel(), s)
            self.xd = xs
        if phases is not None:
            phases[4].record()
        nat.call('somgb_neighbourhood_update_grid', self.S.data_ptr(), self.c.data_ptr(), self.topo.data_ptr(),
                 self.w['m'], self.w['n'], self.D, self.sigma(), self.wnext.data_ptr(), None, None,
                 self.upd_ws.data_ptr(), self.upd_ws.numel(), s)
        if phases is not None:
            phases[3].record()
        self.wcur, self.wnext = self.wnext, self.wcur
        self.epoch += 1

    def rechecks(self):
        v = np.zeros(1, dtype=np.int64)
        self.nat.call('somgb_last_recheck_count', v.ctypes.data, self.t.cuda.current_stream().cuda_stream)
        return int(v[0])


def time_epochs(torch, runner, warmup, steps, sustain_s=0.0):
    """W warm-up epochs, then exactly `steps` epochs between two events (each dominant kernel timed too); then, untimed,
    the same epochs for `sustain_s` seconds more (a window for the clock samples), and one epoch with phase events."""
    errs = torch.zeros((warmup + steps, 3), dtype=torch.float64, device=runner.dev)
    for i in range(warmup):
        runner.step(errs[i])
    torch.cuda.synchronize()
    kt = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    for a, b in kt:          # torch creates the CUDA event at its first record; the library re-records these
        a.record()
        b.record()
    start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    launches0 = runner.nat.lib().somgb_kernel_launches()
    runner.sweep2_log = []
    start.record()
    for i in range(steps):
        runner.step(errs[warmup + i], timer=kt[i])
    stop.record()
    torch.cuda.synchronize()
    launches = runner.nat.lib().somgb_kernel_launches() - launches0
    rechecks = runner.rechecks()
    runner.timed_sweep2 = [int(t.item()) for t in runner.sweep2_log]   # per timed epoch
    total_ms = start.elapsed_time(stop)
    kernel_ms = [a.elapsed_time(b) for a, b in kt]
    extra = torch.zeros(3, dtype=torch.float64, device=runner.dev)
    t_end = time.perf_counter() + sustain_s
    while time.perf_counter() < t_end:
        runner.step(extra)
        torch.cuda.synchronize()
    ph = [torch.cuda.Event(enable_timing=True) for _ in range(5)]
    runner.step(extra, phases=ph)
    torch.cuda.synchronize()
    phases = {'bmu_pass_ms': ph[0].elapsed_time(ph[1]), 'accumulate_ms': ph[1].elapsed_time(ph[2]),
              'regroup_rows_ms': ph[2].elapsed_time(ph[4]), 'neighbourhood_update_ms': ph[4].elapsed_time(ph[3])}
    return total_ms, kernel_ms, launches, errs.cpu().numpy(), phases, rechecks


def find_bmus(torch, native, xd, w, algo):
    N, D = xd.shape
    M = w.shape[0]
    out = torch.empty(N, dtype=torch.int32, device=xd.device)
    nb = native.workspace_bytes(native.OP_FIND_BMUS, N, M, D, native.ALGOS[algo])
    wsb = torch.empty(nb + 256, dtype=torch.uint8, device=xd.device)
    native.call('somgb_find_bmus', xd.data_ptr(), N, D, w.data_ptr(), M, native.ALGOS[algo], out.data_ptr(),
                wsb.data_ptr() + (-wsb.data_ptr()) % 256, nb, torch.cuda.current_stream().cuda_stream)
    del wsb
    return out


def bmu_check(torch, xd, w, bmu, train=False, chunk=1 << 16):
    """BMUs of the tensor-core pass on every row against an independent evaluation: float32 GEMM distances find each
    row's three nearest units, whose distances are then taken in the reference's typing (float32 differences and
    squares, float64 sum) and ranked by (distance, unit). Rows whose two best reference distances lie within the
    float32 rounding bound 2 (D + 2) 2^-24 of each other are near-ties: counted, and adjudicated by float64 distances
    over every unit. A row whose GEMM three do not contain its BMU is scanned in full as well. `train`: BMUs of
    training semantics (-1 for a row without a valid unit)."""
    N, D = xd.shape
    tol = 2.0 * (D + 2) * 2.0 ** -24
    wd = w.double()
    wn = (w * w).sum(1)
    mism = ties = tie_agree = tie_differ = scanned = 0
    for a in range(0, N, chunk):
        x = xd[a:a + chunk]
        dist = (x * x).sum(1, keepdim=True) - 2.0 * (x @ w.T) + wn[None, :]
        top = torch.topk(dist, 3, dim=1, largest=False).indices                      # (b, 3)
        t = w[top] - x[:, None, :]                                                    # float32 differences
        dref = (t * t).double().sum(-1)                                               # float32 squares, float64 sum
        dref = torch.where(torch.isnan(dref), torch.full_like(dref, float('inf')), dref)
        order = torch.argsort(top, dim=1)                                            # unit order, then stable by value
        top = torch.gather(top, 1, order)
        dref = torch.gather(dref, 1, order)
        srt = torch.argsort(dref, dim=1, stable=True)
        d_sorted = torch.gather(dref, 1, srt)
        b_ref = torch.gather(top, 1, srt)[:, 0].to(torch.int32)
        b = bmu[a:a + chunk]
        near = (d_sorted[:, 1] - d_sorted[:, 0]) <= tol * d_sorted[:, 0]
        in_top = (top == b[:, None].long()).any(1)
        full = near | ~in_top | ~torch.isfinite(d_sorted[:, 0])
        ok = (b == b_ref) | full
        if train:
            ok = ok | (b < 0)
        mism += int((~ok).sum().item())
        idx = torch.nonzero(full & (b >= 0) if train else full).flatten()
        scanned += int(idx.numel())
        for k in range(0, int(idx.numel()), 256):
            # float64 distances over every unit (the adjudication) and the reference-typed argmin (full scan)
            ii = idx[k:k + 256]
            xs = x[ii]
            d64 = ((wd[None, :, :] - xs.double()[:, None, :]) ** 2).sum(-1)
            b64 = torch.argmin(torch.nan_to_num(d64, nan=float('inf')), dim=1).to(torch.int32)
            t32 = w[None, :, :] - xs[:, None, :]
            dr = (t32 * t32).double().sum(-1)
            b_full = torch.argmin(torch.nan_to_num(dr, nan=float('inf')), dim=1).to(torch.int32)
            bb = b[ii]
            mism += int((bb != b_full).sum().item())
            nt = near[ii]
            ties += int(nt.sum().item())
            tie_agree += int(((bb == b64) & nt).sum().item())
            tie_differ += int(((bb != b64) & nt).sum().item())
    return {'rows': int(N), 'mismatches_vs_reference_typing': mism, 'near_ties': ties, 'near_tie_tol_rel': tol,
            'near_ties_fp64_agrees': tie_agree, 'near_ties_fp64_differs': tie_differ, 'rows_scanned_in_full': scanned,
            'how': 'float32 GEMM top-3 per row, then the reference typing (float32 squares, float64 sum) and '
                   '(distance, unit) order; near-ties and rows outside the top-3 scanned over every unit; near-ties '
                   'adjudicated by float64 distances'}


def weights_check(torch, runner):
    """One more epoch of the runner, then its new weights against a float64 evaluation of the same update: the per-BMU
    sums S, c of the epoch's own BMUs in float64, num = H S and den = H c with the reference's neighbourhood factor
    h_jb = exp(-|t_j - t_b|^2 / (2 sigma^2)) (|t_j - t_b|^2 typed as the reference: float32 differences and squares,
    float64 sum), w = num / den where den > 1e-12."""
    sigma = runner.sigma()
    extra = torch.zeros(3, dtype=torch.float64, device=runner.dev)
    runner.step(extra)
    torch.cuda.synchronize()
    w32 = runner.wcur.double()
    keep = runner.bmu >= 0
    b = runner.bmu[keep].long()
    S = torch.zeros((runner.M, runner.D), dtype=torch.float64, device=runner.dev)
    S.index_add_(0, b, runner.x_pass[keep].double())
    c = torch.bincount(b, minlength=runner.M).double()
    s_rel = float(((runner.S - S).abs().max() / S.abs().max().clamp_min(1e-300)).item())
    t = runner.topo
    d = t[:, None, :] - t[None, :, :]
    d2 = (d * d).double().sum(-1)
    H = torch.exp(-d2 / (2.0 * sigma * sigma))
    num = H @ S
    den = H @ c
    w64 = torch.where(den[:, None] > 1e-12, num / den[:, None], torch.zeros_like(num))
    rel = (w32 - w64).abs() / w64.abs().clamp_min(1e-30)
    rel = torch.where(w64 == 0, (w32 - w64).abs(), rel)
    return {'max_rel': float(rel.max().item()), 'rms_rel': float(rel.pow(2).mean().sqrt().item()),
            'sums_max_rel': s_rel, 'epoch_sigma': sigma, 'rows': runner.N,
            'against': 'a float64 evaluation of the same epoch update (float64 per-BMU sums of the same BMUs, '
                       'pairwise Gaussian contraction, divide)'}


def fp32_roofline(N, M, D, ms, clocks):
    """The plain FP32 form's BMU pass against the nominal FP32 FMA rate of the part (SMs x 128 lanes x 2 flops at the
    sampled maximum SM clock): algorithmic 2 N M D flops of direct differences."""
    import torch
    sms = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
    mhz = (clocks or {}).get('sm_max_mhz') or 2070.0
    peak = sms * 128 * 2 * mhz * 1e6 / 1e12
    ach = 2.0 * N * M * D / (ms * 1e-3) / 1e12
    return {'achieved': ach, 'peak': peak, 'unit': 'TFLOP/s', 'frac': ach / peak,
            'peak_source': f'nominal FP32 FMA rate: {sms} SMs x 128 lanes x 2 flops x {mhz:.0f} MHz'}


def iteration_record(torch, native, xd, wmap, topo, w, device):
    """Iteration mode (SOM_Batch.train(n_vectors=N)'s pass, algo/som_batch.py:154-210, 378-495) on the resident
    catalogue and the trained map: one somgb_train_iter_pass_grid over every row on the tensor cores (BMU pass and the
    contraction) and on the CUDA cores (float32 BMU search and contraction), CUDA-event timed, with the BMU pass alone
    timed to give the contraction's share, and the largest relative difference of the two forms' sums."""
    N, D = xd.shape
    m, n = w['m'], w['n']
    M = m * n
    s = torch.cuda.current_stream(device).cuda_stream
    out = {'call': f'somgb_train_iter_pass_grid(all {N} rows, cur_vector 0, n_vectors {N}, sigma0 {w["sigma0"]})',
           'unit': UNIT}
    sums = {}
    for algo in ('tc', 'fp32'):
        A = native.ALGOS[algo]
        nbytes = native.workspace_bytes(native.OP_EPOCH, N, M, D, A)
        buf = torch.empty(nbytes + 256, dtype=torch.uint8, device=device)
        wsp = buf.data_ptr() + (-buf.data_ptr()) % 256
        num = torch.zeros((M, D), dtype=torch.float64, device=device)
        den = torch.zeros(M, dtype=torch.float64, device=device)
        bmu = torch.empty(N, dtype=torch.int32, device=device)

        def whole():
            num.zero_()
            den.zero_()
            native.call('somgb_train_iter_pass_grid', xd.data_ptr(), None, N, D, wmap.data_ptr(), topo.data_ptr(), m,
                        n, float(w['sigma0']), 0, N, A, num.data_ptr(), den.data_ptr(), wsp, nbytes, s)

        def bmus():
            native.call('somgb_train_bmu_pass', xd.data_ptr(), None, N, D, wmap.data_ptr(), topo.data_ptr(), M, 1.0,
                        A, bmu.data_ptr(), None, wsp, nbytes, s)

        ms = {}
        for label, fn in (('pass', whole), ('bmu', bmus)):
            for _ in range(2):
                fn()
            torch.cuda.synchronize()
            ts = []
            for _ in range(3):
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record()
                fn()
                e1.record()
                torch.cuda.synchronize()
                ts.append(e0.elapsed_time(e1))
            ms[label] = statistics.mean(ts)
        whole()
        torch.cuda.synchronize()
        sums[algo] = (num.clone(), den.clone())
        key = 'tensor_cores' if algo == 'tc' else 'cuda_cores'
        out[key] = {'ms_per_pass': ms['pass'], 'bmu_pass_ms': ms['bmu'], 'contraction_ms': ms['pass'] - ms['bmu'],
                    'value': N * M / (ms['pass'] * 1e-3) / 1e9,
                    'contraction': 'tcgen05 split-FP16 (k4_iter_kernel)' if algo == 'tc' else
                                   'float32 CUDA cores (iter_grid_kernel)'}
        del buf, num, den, bmu
    (nt, dt), (nf, df) = sums['tc'], sums['fp32']
    out['value'] = out['tensor_cores']['value']
    out['contraction_speedup'] = out['cuda_cores']['contraction_ms'] / out['tensor_cores']['contraction_ms']
    out['max_rel_diff_den'] = float(((dt - df).abs() / df.abs().clamp_min(1e-9 * float(df.abs().max()))).max())
    out['max_rel_diff_num'] = float(((nt - nf).abs() / (nf.abs() + 1e-6 * float(nf.abs().max()))).max())
    return out


def sq64_record(torch, native, device, args):
    """The 64x64, D = 32 configuration over 50.3 M rows, catalogue generated on the device: tensor-core epochs, the
    plain FP32 form's epochs, the recheck rate and BMU mismatches between the two forms on the final map."""
    import decontamination_gb300 as dg
    from decontamination_gb300 import synthetic
    w = WORKLOADS['sq64']
    M, D, N = w['m'] * w['n'], w['d'], w['N']
    xd = synthetic.correlated_lognormal_device(N, D, w['seed'], device)
    w0 = synthetic.uniform_weights(M, D, w['seed'])
    topo = torch.from_numpy(dg.SOM_Batch(w['m'], w['n'], D, topology=w['topology'])._topography).to(device)
    out = {'workload': w['name'], 'N': N, 'M': M, 'D': D,
           'data': 'synthetic on the device (the correlated log-normal recipe, torch generator)'}
    r = EpochRunner(torch, native, xd, w0, topo, w, 'auto', device)
    # the headline's window: epochs 3 to 22, the whole 20-epoch schedule once
    steps = 20
    total, kms, _, _, ph, rc = time_epochs(torch, r, 3, steps)
    out.update({'value': N * M / (total / steps * 1e-3) / 1e9, 'ms_per_step': total / steps, 'epochs_timed': steps,
                'bmu_kernel_ms': statistics.mean(kms), 'phases': ph, 'recheck_rows_last_epoch': rc,
                'recheck_rate': rc / N})
    wfin = r.wcur.clone()
    del r
    torch.cuda.empty_cache()
    if not args.skip_fp32:
        r32 = EpochRunner(torch, native, xd, w0, topo, w, 'fp32', device)
        t32, k32, _, _, _, _ = time_epochs(torch, r32, 1, 2)
        del r32
        out['fp32_form'] = {'value': N * M / (t32 / 2 * 1e-3) / 1e9, 'ms_per_step': t32 / 2,
                            'bmu_kernel_ms': statistics.mean(k32)}
        out['speedup_vs_fp32_form'] = out['fp32_form']['ms_per_step'] / out['ms_per_step']
        b_tc = find_bmus(torch, native, xd, wfin, 'tc')
        b_32 = find_bmus(torch, native, xd, wfin, 'fp32')
        out['bmu_mismatches_vs_fp32_form'] = int((b_tc != b_32).sum().item())
        del b_tc, b_32
    del xd
    torch.cuda.empty_cache()
    return out


def gpu_arm(args, ws, rank, local):
    import torch
    import torch.distributed as dist
    from decontamination_gb300 import build as gbuild, _native
    import decontamination_gb300 as dg

    gbuild.build()
    torch.cuda.set_device(local)
    torch.backends.cuda.matmul.allow_tf32 = False
    device = torch.device('cuda', local)
    if ws > 1:
        dist.init_process_group('nccl', device_id=device)
    w = WORKLOADS[args.workload]
    M, D = w['m'] * w['n'], w['d']
    x, w0 = make_data(args.n or w['N'], w)
    N = x.shape[0]
    topo_np = dg.SOM_Batch(w['m'], w['n'], D, topology=w['topology'])._topography
    xh = torch.from_numpy(x).pin_memory()
    xd = xh.to(device)
    topo = torch.from_numpy(topo_np).to(device)

    def barrier():
        if ws > 1:
            dist.barrier()
        torch.cuda.synchronize()

    # --- main: epochs with the catalogue resident ---------------------------------------------------------------------
    runner = EpochRunner(torch, _native, xd, w0, topo, w, args.algo, device)
    used_algo = 'tc' if _native.workspace_bytes(_native.OP_FIND_BMUS, N, M, D, _native.ALGO_TC) > 256 and \
        args.algo != 'fp32' else 'fp32'
    barrier()
    with ClockSampler(gpu_bus_id(torch, device)) as clk:
        total_ms, kernel_ms, launches, errs, phases, rechecks = time_epochs(torch, runner, args.warmup, args.steps,
                                                                            args.clock_seconds)
    barrier()
    clocks = clk.summary()
    clocks['window'] = f'the {args.steps} timed epochs and {args.clock_seconds:.1f} s more of the same epochs'
    ms_per_step = slowest_rank(total_ms, ws, device) / args.steps
    value = whole_job_rate(ws, N, M, ms_per_step)

    # roofline of the dominant kernel (the BMU pass): algorithmic 2*N*M*D flops per launch
    peaks, peak_kind = measured_peaks()
    k_ms = statistics.mean(kernel_ms)
    flops = 2.0 * N * M * D
    achieved_tflops = flops / (k_ms * 1e-3) / 1e12
    peak = peaks.get('bf16_tflops_sustained', peaks.get('bf16_tflops'))
    traffic = K1_DRAM_BYTES_PER_ROW.get(args.workload)
    roofline = {'bound': 'tensor', 'achieved': achieved_tflops, 'peak': peak, 'unit': 'TFLOP/s',
                'frac': achieved_tflops / peak,
                'traffic': traffic * N if (traffic and used_algo == 'tc') else None,
                'traffic_source': 'ncu dram__bytes_read.sum + dram__bytes_write.sum of the 4,194,304-row case of this '
                                  'workload, scaled by rows' if traffic else None,
                'kernel': 'BMU pass (%s)' % ('tcgen05 split-FP16' if used_algo == 'tc' else 'FP32 CUDA cores'),
                'kernel_ms': k_ms, 'kernel_share': k_ms * args.steps / total_ms,
                'peak_source': f'{peak_kind} bf16_tflops_sustained (dense FP16 and BF16 share the rate)',
                'hbm_bytes_algorithmic': N * D * 4 + N * 4,
                'hbm_frac': (N * D * 4 + N * 4) / (k_ms * 1e-3) / 1e9 / peaks.get('hbm_gbs', 6800.0)}
    if used_algo == 'tc':
        # What the tensor pipe executes: 128-row x 256-unit column tiles of the split-FP16 contraction, K = 16 x K-steps
        # (lo.hi, hi.lo, hi.hi blocks and the |w|^2 step); sweep 1 computes every column tile of each row tile, sweep 2
        # those with a candidate (counted by the pass).
        k_steps = 3 * (D // 16) + 1 if D % 16 == 0 else (3 * D + 2 + 15) // 16
        row_tiles, col_tiles = (N + 127) // 128, (M + 255) // 256
        sweep2 = statistics.mean(runner.timed_sweep2)
        tiles = row_tiles * col_tiles + sweep2
        executed = tiles * 2.0 * 128 * 256 * (16 * k_steps) / (k_ms * 1e-3) / 1e12
        roofline['executed_tensor_tflops'] = executed
        roofline['executed_frac'] = executed / peak
        roofline['column_tiles_per_row_tile'] = {'sweep1': col_tiles, 'sweep2': sweep2 / row_tiles}
    out = {
        'metric': METRIC, 'value': value, 'unit': UNIT, 'n_gpus': ws, 'steps': args.steps, 'warmup': args.warmup,
        'ms_per_step': ms_per_step, 'higher_is_better': True, 'scaling': 'weak', 'vs_baseline': None,
        'dtype': 'f16x3-split/f32acc' if used_algo == 'tc' else 'f32',
        'data': 'synthetic (seeded correlated log-normal, cond 100, 2% rows x10; weights U[-1,1])',
        'config': {'workload': w['name'], 'algo': used_algo, 'N_per_gpu': N, 'M': M, 'D': D,
                   'l2': f'catalogue {N * D * 4 / 1e6:.0f} MB > 129 MB L2 per epoch; no flush',
                   'parallelism': f'replicas x{ws}'},
        'roofline': roofline, 'gpu_launches': int(launches), 'clocks': clocks, 'phases': phases,
        'recheck_last_epoch': rechecks,
        'qe_last': float(errs[-1][0] / errs[-1][2]) if errs[-1][2] > 0 else None,
    }

    # --- plain FP32 form of the same epoch ------------------------------------------------------------------------------
    if not args.skip_fp32 and used_algo == 'tc':
        r32 = EpochRunner(torch, _native, xd, w0, topo, w, 'fp32', device)
        n32 = max(3, args.steps // 4)
        t32, k32, _, _, ph32, _ = time_epochs(torch, r32, min(args.warmup, 3), n32)
        del r32
        out['fp32_form'] = {'value': N * M / (t32 / n32 * 1e-3) / 1e9, 'ms_per_step': t32 / n32,
                            'bmu_kernel_ms': statistics.mean(k32), 'phases': ph32,
                            'roofline': fp32_roofline(N, M, D, statistics.mean(k32), clocks)}
        out['speedup_vs_fp32_form'] = out['fp32_form']['ms_per_step'] / ms_per_step
        # matched BMUs: both forms on the tensor-core run's final map, every row of the catalogue
        b_tc = find_bmus(torch, _native, xd, runner.wcur, 'tc')
        b_32 = find_bmus(torch, _native, xd, runner.wcur, 'fp32')
        out['fp32_form']['bmu_mismatches'] = int((b_tc != b_32).sum().item())
        out['fp32_form']['bmu_rows_compared'] = N
        del b_tc, b_32

    # --- parity at full size: BMUs against an independent evaluation, weights against float64 ---------------------------
    if not args.skip_parity:
        b = find_bmus(torch, _native, xd, runner.wcur, args.algo)
        out['parity'] = {'bmu': bmu_check(torch, xd, runner.wcur, b)}
        del b
        out['parity']['weights'] = weights_check(torch, runner)
        torch.cuda.empty_cache()

    # --- end to end through the public API ------------------------------------------------------------------------------
    if not args.skip_e2e:
        som = dg.SOM_Batch(w['m'], w['n'], D, topology=w['topology'], sigma=w['sigma0'])
        som.bmu_algo = args.algo
        e2e_steps = max(1, min(args.steps, 5))
        for _ in range(3):                                      # warm-up (allocations, library state)
            som._weights[...] = w0
            som.train(xh, n_epochs=1, use_best_epoch=False)
        gc.collect()   # no pending collection of the earlier records' objects lands in the timed calls
        barrier()
        t0 = time.perf_counter()
        calls = []
        for _ in range(e2e_steps):
            tc0 = time.perf_counter()
            som._weights[...] = w0
            som.train(xh, n_epochs=1, use_best_epoch=False)
            calls.append((time.perf_counter() - tc0) * 1e3)
        barrier()
        dt = slowest_rank((time.perf_counter() - t0) / e2e_steps, ws, device)
        h2d = x.nbytes + w0.nbytes + topo_np.nbytes
        d2h = 2 * w0.nbytes + 3 * 8 * 2
        out['e2e'] = {'value': whole_job_rate(ws, N, M, dt * 1e3), 'unit': UNIT, 'h2d_bytes_per_step': h2d,
                      'd2h_bytes_per_step': d2h, 'ms_per_step': dt * 1e3, 'calls_ms': [round(v, 2) for v in calls],
                      'call': 'SOM_Batch.train(pinned host tensor, n_epochs=1): upload, training pass, error pass, '
                              'weights/history/errors back to the host'}
        del som

    # --- BMU serving (rank 0, one GPU), before the other sub-records' large buffers come and go --------------------------
    if not args.skip_serve and rank == 0 and ws == 1:
        out['serve'] = serve_record(args)
        torch.cuda.empty_cache()

    # --- iteration mode on the resident catalogue and the trained map (rank 0, one GPU) --------------------------------------
    if not args.skip_iter and rank == 0 and ws == 1 and w['topology'] in ('square', 'hexagonal'):
        out['iteration'] = iteration_record(torch, _native, xd, runner.wcur, topo.float(), w, device)
        torch.cuda.empty_cache()

    del runner, xd
    torch.cuda.empty_cache()

    # --- the 64x64, D = 32 configuration (rank 0, one GPU) ---------------------------------------------------------------
    if not args.skip_sq64 and rank == 0 and ws == 1 and args.n is None:
        out['sq64'] = sq64_record(torch, _native, device, args)

    # --- CPU baseline (rank 0, N=1) -------------------------------------------------------------------------------------
    if not args.skip_cpu and rank == 0 and ws == 1:
        r, ns, nt, dt = cpu_epoch_rate(x, w0, w, seconds=args.cpu_seconds)
        out['cpu_baseline'] = {'value': r, 'unit': UNIT, 'cores': nt, 'kind': 'port',
                               'sample': f'first {ns} rows of the workload, one reference-formulation epoch '
                                         f'(scatter + float32 atomics) and its error pass, {dt:.1f} s'}
    if rank == 0:
        print(json.dumps(out), flush=True)
    if ws > 1:
        dist.barrier()
        dist.destroy_process_group()


# ----------------------------------------------------------------------------------------------------------------------
# BMU serving: requests of mixed sizes on a resident 64x64 map
# ----------------------------------------------------------------------------------------------------------------------

SERVE = dict(name='BMU serving: square 64x64 map (M = 4096), D = 16, Poisson arrivals, request sizes log-uniform '
                  'in [1e3, 1e7] rows', m=64, n=64, d=16, seed=4, pool=10_000_000, lo=1_000, hi=10_000_000)


def serve_record(args):
    """Requests arrive as a Poisson process and are submitted to SomServer as slices of a pinned host catalogue;
    latency is submit to result on the host. The map is trained once (3 epochs on 500k rows) before the clock runs."""
    import threading
    import torch
    import decontamination_gb300 as dg
    from decontamination_gb300 import synthetic, _native, build as gbuild
    from decontamination_gb300.serve import SomServer
    gbuild.build()
    s = SERVE
    M, D = s['m'] * s['n'], s['d']
    pool = torch.from_numpy(synthetic.gaussian_mixture(s['pool'], D, s['seed'])).pin_memory()
    som = dg.SOM_Batch(s['m'], s['n'], D, topology='square')
    som.init_rand(seed=s['seed'])
    som.bmu_algo = args.algo
    som.train(pool[:500_000].numpy(), n_epochs=3)
    algo_used = 'tc' if _native.lib().somgb_algo_supported(_native.ALGO_TC, s['pool'], M, D) and \
        args.algo != 'fp32' else 'fp32'
    rng = np.random.default_rng(s['seed'])
    n_req = max(1, int(rng.poisson(args.serve_rate * args.serve_seconds)))
    arrivals = np.sort(rng.uniform(0.0, args.serve_seconds, n_req))
    sizes = np.exp(rng.uniform(np.log(s['lo']), np.log(s['hi']), n_req)).astype(np.int64)
    starts = rng.integers(0, s['pool'] - sizes + 1)
    with SomServer(max_batch_rows=1 << 20) as srv:
        mid = srv.add_map(som)
        # warm-up: every request shape class once (library state, pinned staging buffers), then two requests of the
        # largest size together, so that both workers hold buffers for it before the clock runs
        for n in (1_000, 100_000, 2_000_000):
            srv.submit_bmu(mid, pool[:n], histogram=True).result()
        big = [srv.submit_bmu(mid, pool[:s['hi']], histogram=True) for _ in range(2)]
        for f in big:
            f.result()
        futs = [None] * n_req
        t0 = time.perf_counter()

        def feeder():
            for i in range(n_req):
                delay = t0 + arrivals[i] - time.perf_counter()
                if delay > 0:
                    time.sleep(delay)
                futs[i] = srv.submit_bmu(mid, pool[starts[i]:starts[i] + sizes[i]], histogram=True)

        th = threading.Thread(target=feeder)
        th.start()
        th.join()
        for f in futs:
            f.result()
        t_end = time.perf_counter()
    # latencies of the timed requests only (the five warm-up requests completed first)
    lat = np.asarray(srv.latencies('bmu')[5:]) * 1e3
    rows = int(sizes.sum())
    wall = t_end - t0
    return {
        'workload': s['name'], 'p50_ms': float(np.percentile(lat, 50)), 'p99_ms': float(np.percentile(lat, 99)),
        'mean_ms': float(lat.mean()), 'requests': n_req, 'rows': rows, 'wall_s': wall,
        'throughput': {'value': rows * M / wall / 1e9, 'unit': UNIT},
        'offered': {'requests_per_s': args.serve_rate, 'sample_units_per_s': rows * M / args.serve_seconds / 1e9,
                    'unit': UNIT, 'window_s': args.serve_seconds},
        'passes': len(srv.batch_sizes()), 'algo': algo_used, 'workers': srv.workers, 'max_batch_rows': 1 << 20,
        'returns': 'int32 BMUs + M-bin activation histogram per request',
        'data': 'synthetic (seeded 5-component Gaussian mixture, D = 16); requests are slices of a pinned 1e7-row '
                'catalogue'}


def serve_arm(args):
    r = serve_record(args)
    out = {'metric': 'BMU-serve latency p99', 'value': r['p99_ms'], 'unit': 'ms', 'higher_is_better': False,
           'n_gpus': 1, **r}
    print(json.dumps(out), flush=True)


MIXED = dict(name='mixed-training serving: grids uniform in {8x8, 16x16, 32x32, 48x48, 80x80}, square or hexagonal, '
                  'D in {4, 8, 16, 32}, N log-uniform in [1e4, 5e6], 5-component Gaussian mixture or correlated '
                  'log-normal, 10-30 epochs, weights U[-1, 1]', grids=(8, 16, 32, 48, 80), dims=(4, 8, 16, 32),
             lo=10_000, hi=5_000_000, seed=5)


def mixed_jobs(n_jobs):
    """The seeded job list of the mixed-training workload (one dict per job)."""
    c = MIXED
    rng = np.random.default_rng(c['seed'])
    jobs = []
    for i in range(n_jobs):
        g = int(rng.choice(c['grids']))
        jobs.append(dict(m=g, n=g, topology=str(rng.choice(['square', 'hexagonal'])), d=int(rng.choice(c['dims'])),
                         N=int(np.exp(rng.uniform(np.log(c['lo']), np.log(c['hi'])))),
                         gen=str(rng.choice(['mixture', 'lognormal'])), epochs=int(rng.integers(10, 31)),
                         seed=1000 + i))
    return jobs


def serve_train_record(args, algo):
    """All jobs are submitted to SomServer as they are generated (each catalogue made on the device, then handed to
    the server), trained on its two training streams under its device-memory admission; completion latency is from
    submission to the trained map on the host."""
    import torch
    import decontamination_gb300 as dg
    from decontamination_gb300 import synthetic
    from decontamination_gb300.serve import SomServer
    device = torch.device('cuda', torch.cuda.current_device())
    jobs = mixed_jobs(args.jobs)
    futs, work = [], 0
    with SomServer(train_workers=2) as srv:
        # warm-up: one small job of every D (library state, workspaces)
        for d in MIXED['dims']:
            som = dg.SOM_Batch(8, 8, d, topology='square')
            som.bmu_algo = algo
            srv.submit_train(som, synthetic.gaussian_mixture_device(20_000, d, 1, device), n_epochs=2).result()
        n_warm = len(srv.latencies('train'))
        t0 = time.perf_counter()
        for j in jobs:
            gen = synthetic.gaussian_mixture_device if j['gen'] == 'mixture' else \
                synthetic.correlated_lognormal_device
            x = gen(j['N'], j['d'], j['seed'], device)
            torch.cuda.current_stream().synchronize()
            som = dg.SOM_Batch(j['m'], j['n'], j['d'], topology=j['topology'])
            som._weights[...] = synthetic.uniform_weights(j['m'] * j['n'], j['d'], j['seed']).reshape(
                som._weights.shape)
            som.bmu_algo = algo
            futs.append(srv.submit_train(som, x, n_epochs=j['epochs'], use_best_epoch=False))
            work += j['N'] * j['m'] * j['n'] * j['epochs']
            del x
        for f in futs:
            f.result()
        wall = time.perf_counter() - t0
        lat = np.asarray(srv.latencies('train')[n_warm:]) * 1e3
    return {'algo': algo, 'jobs': len(jobs), 'jobs_per_s': len(jobs) / wall, 'wall_s': wall,
            'p50_ms': float(np.percentile(lat, 50)), 'p99_ms': float(np.percentile(lat, 99)),
            'epoch_sample_units_per_s': {'value': work / wall / 1e9, 'unit': UNIT}}


def serve_train_arm(args):
    from decontamination_gb300 import build as gbuild
    gbuild.build()
    recs = [serve_train_record(args, a.strip()) for a in args.train_algos.split(',') if a.strip()]
    jobs = mixed_jobs(args.jobs)
    out = {'metric': 'mixed-training serving jobs/s', 'value': recs[0]['jobs_per_s'], 'unit': 'jobs/s',
           'higher_is_better': True, 'n_gpus': 1, 'workload': MIXED['name'], 'runs': recs,
           'jobs': {'count': len(jobs), 'rows_total': int(sum(j['N'] for j in jobs)),
                    'tensor_core_jobs': int(sum(1 for j in jobs if j['m'] * j['n'] >= 32 and
                                                j['N'] * j['m'] * j['n'] >= (1 << 22))),
                    'sample_unit_epochs': float(sum(j['N'] * j['m'] * j['n'] * j['epochs'] for j in jobs))},
           'data': 'synthetic, generated on the device per job (seeded)'}
    if len(recs) > 1:
        out['speedup_vs_' + recs[1]['algo']] = recs[0]['jobs_per_s'] / recs[1]['jobs_per_s']
    print(json.dumps(out), flush=True)


def main():
    args = parse()
    ws, rank, local = dist_env()
    if args.serve:
        if rank == 0:
            serve_arm(args)
        return
    if args.serve_train:
        if rank == 0:
            serve_train_arm(args)
        return
    if args.impl == 'reference':
        reference_arm(args, ws, rank)
    else:
        gpu_arm(args, ws, rank, local)


if __name__ == '__main__':
    main()
