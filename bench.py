"""Benchmark: CPAB transform_data forward + backward (dtheta and d(data)).

Workload (the configuration the headline metric is quoted on): 2D
tessellation [3,3] with zero boundary (d = 34), 64 theta ~ N(0, 0.5^2 I), data
[64, 3, 224, 224] uniform[0,1] smoothed by a 5x5 box filter, transform_data on
a 224x224 grid, loss = MSE against the same images warped by a second theta.
One step = forward + backward of that loss over the whole batch
(64 * 224 * 224 = 3,211,264 point trajectories of 50 steps).  Metric: points/s.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl {gb300,reference}]

Under torchrun (N > 1) every rank runs the full batch with its own seeds
(weak scaling, no data-path collective); the slowest rank's time sets the
aggregate.  --impl reference times the reference's CPU implementation of the
same step (its compiled libcpab/core/cpab_ops.cpp op, all host threads; the C
restatement only where that build is missing) on a bounded sample.  Beside the
headline the line carries the reference's own GPU path on the same inputs
(plain_gpu_reference), the timed step's error against the FP64 oracle
(error_vs_fp64), the autotuned launch shapes and the other workloads' legs.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np
import torch
import torch.nn.functional as F

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

METRIC = 'points/s fwd+dθ bwd, 2D 3×3 224² b64: fused vs plain GPU, err≤1e-5 vs FP64'
NC = [3, 3]
BATCH, SIZE, CHANNELS, NSTEPS = 64, 224, 3, 50
THETA_STD = 0.5
L2_BYTES = 129 * 2 ** 20
# algorithmic work per point trajectory (2D, 50 steps): forward 17 flop/step,
# adjoint 37 flop/step; interpolation 8*C bytes (forward), 12*C (backward)
FLOP_FWD_STEP, FLOP_ADJ_STEP = 17, 37
# thread instructions per point-step of the fused kernels (2D [3,3], reference
# gradient), from the ncu capture of 16 images summarised in profiles/
# (smsp__inst_executed x active threads per instruction / point-steps)
INSTR_FWD_STEP, INSTR_BWD_STEP = 73, 216
# DRAM bytes (read + write) of one k_transform_data_backward launch per image,
# from an ncu capture of 16 images (36.26 MB); traffic grows with the images
# processed
BWD_DRAM_BYTES_PER_IMAGE = 36.26e6 / 16


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument('--gpus', type=int, default=1)
    ap.add_argument('--steps', type=int, default=20)
    ap.add_argument('--warmup', type=int, default=5)
    ap.add_argument('--impl', default='gb300', choices=['gb300', 'reference'])
    ap.add_argument('--cpu-sample-images', type=int, default=CPU_SAMPLE_IMAGES)
    ap.add_argument('--batch', type=int, default=BATCH,
                    help='images per step (the headline workload uses 64; smaller values '
                         'are for profiling runs only)')
    ap.add_argument('--no-cpu-baseline', action='store_true')
    ap.add_argument('--leg', default='all',
                    choices=['all', 'ragged', 'volume', 'interp', 'aligner', 'exact', 'points',
                             'mixed', 'plain', 'cfg1', 'cfg5'],
                    help='run only one of the side workloads and print its result (for '
                         'profiling runs)')
    ap.add_argument('--no-tune', action='store_true',
                    help='use the built-in launch heuristics instead of autotuning the '
                         'launch shapes')
    ap.add_argument('--no-plain', action='store_true',
                    help="skip the reference's own GPU path (the plain comparator)")
    ap.add_argument('--no-extra', action='store_true',
                    help='skip the workloads reported beside the headline (ragged 1D '
                         'series, 3D volume warp, interpolator sweep)')
    args = ap.parse_args()
    return args


def dist_env():
    rank = int(os.environ.get('RANK', '0'))
    world = int(os.environ.get('WORLD_SIZE', '1'))
    local = int(os.environ.get('LOCAL_RANK', '0'))
    return rank, world, local


def make_inputs(T, device, seed_offset=0, batch=BATCH):
    d = T.get_theta_dim()
    BATCH = batch
    g0 = torch.Generator().manual_seed(0 + seed_offset)
    g1 = torch.Generator().manual_seed(1 + seed_offset)
    g2 = torch.Generator().manual_seed(2 + seed_offset)
    theta = THETA_STD * torch.randn(BATCH, d, generator=g0)
    raw = torch.rand(BATCH, CHANNELS, SIZE, SIZE, generator=g1)
    data = F.avg_pool2d(raw, kernel_size=5, stride=1, padding=2, count_include_pad=False)
    theta2 = THETA_STD * torch.randn(BATCH, d, generator=g2)
    with torch.no_grad():
        target = T.transform_data(data.to(device), theta2.to(device), [SIZE, SIZE])
    return theta, data.contiguous(), target.cpu().contiguous()


class ClockSampler:
    """nvidia-smi clock / throttle-reason samples while the timed region runs."""
    FIELDS = ('clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,'
              'clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,'
              'clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap')

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ['nvidia-smi', '-i', str(self.index), '--query-gpu=' + self.FIELDS,
                 '--format=csv,noheader,nounits', '-lms', '100'],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, ValueError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.thread.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ['hw_slowdown', 'hw_thermal_slowdown', 'sw_thermal_slowdown', 'sw_power_cap']
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(',')]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                smax.append(float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[4:8]):
                if v.lower() == 'active':
                    reasons.add(nm)
        if not sm:
            return None
        return {'sm_mhz': statistics.median(sm), 'sm_max_mhz': max(smax),
                'reasons': sorted(reasons), 'samples': len(sm)}


def reduce_max(values, device):
    """Element-wise max over ranks (the slowest rank sets the job time)."""
    import torch.distributed as dist
    t = torch.tensor(values, dtype=torch.float64, device=device)
    if dist.is_available() and dist.is_initialized() and dist.get_world_size() > 1:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return t.tolist()


def time_events(fn, steps, flush=None, stream=None):
    """Per-iteration CUDA-event times (ms) on the launching stream; L2 flushed
    before each iteration outside the timed window."""
    stream = stream or torch.cuda.current_stream()
    times = []
    for _ in range(steps):
        if flush is not None:
            flush()
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        fn()
        b.record(stream)
        b.synchronize()
        times.append(a.elapsed_time(b))
    return times


def workload_config(batch):
    """The headline workload, shared by both arms' JSON lines."""
    return {'workload': 'transform_data 2D tess [3,3] zero_boundary, 64 theta ~ N(0,0.25I), '
                        'data [64,3,224,224] box-filtered U[0,1], MSE vs second warp, '
                        'fwd + dtheta/d(data) bwd',
            'tess_size': NC, 'batch': batch, 'outsize': [SIZE, SIZE], 'nstepsolver': NSTEPS,
            'gradient': 'reference'}


def run_gb300(args):
    from libcpab_gb300 import Cpab, _native as N
    from libcpab_gb300.functions import basis_on
    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group('nccl')
    device = torch.device('cuda', local)
    torch.cuda.set_device(device)
    T = Cpab(NC, backend='pytorch', device='gpu', zero_boundary=True)
    theta_h, data_h, target_h = make_inputs(T, device, seed_offset=10 * rank, batch=args.batch)
    theta_h, data_h, target_h = theta_h.pin_memory(), data_h.pin_memory(), target_h.pin_memory()
    theta = theta_h.to(device)
    data = data_h.to(device)
    target = target_h.to(device)
    flush_buf = torch.empty(2 * L2_BYTES // 4, dtype=torch.float32, device=device)
    flush = lambda: flush_buf.fill_(1.0)

    def step():
        th = theta.detach().requires_grad_(True)
        dd = data.detach().requires_grad_(True)
        out = T.transform_data(dd, th, [SIZE, SIZE])
        loss = F.mse_loss(out, target)
        loss.backward()
        return loss, th.grad, dd.grad

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
            torch.cuda.synchronize()

    # launch shapes of the two fused kernels: autotuned on the timed inputs
    # before anything is timed (the kept shapes serve every later call)
    shapes = None if args.no_tune else tune_headline(T, theta, data, device, flush)
    for _ in range(args.warmup):
        step()
    barrier()
    clocks = ClockSampler(local) if rank == 0 else None
    if clocks:
        clocks.start()
    times_eager = time_events(step, args.steps, flush)
    # the same step (forward, MSE, backward through the public API) captured
    # once in a CUDA graph and replayed: no host work or launch gaps per step
    side = torch.cuda.Stream()
    side.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(side):
        for _ in range(3):
            step()
    torch.cuda.current_stream().wait_stream(side)
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph):
        g_loss, g_dth, g_dd = step()
    for _ in range(args.warmup):
        graph.replay()
    barrier()
    times = time_events(graph.replay, args.steps, flush)
    barrier()
    ms_step = sum(times) / len(times)
    ms_eager = sum(times_eager) / len(times_eager)
    # the replayed graph computes what the eager step computes
    e_loss, e_dth, e_dd = step()
    torch.cuda.synchronize()
    graph_matches = bool(torch.equal(g_dth, e_dth) and torch.equal(g_loss, e_loss))

    # e2e through the public API with host buffers: H2D inputs, D2H loss + dtheta.
    # transform_data_from_host copies the images on a side stream while the
    # trajectories are integrated; the target follows on the same copy stream
    from libcpab_gb300.host_io import HostUpload

    def step_e2e():
        th = theta_h.to(device, non_blocking=True).requires_grad_(True)
        out, dd = T.transform_data_from_host(data_h, th, [SIZE, SIZE], requires_grad=True)
        tg = HostUpload(target_h, device).wait()
        loss = F.mse_loss(out, tg)
        loss.backward()
        res = torch.cat([loss.detach().reshape(1), th.grad.reshape(-1)]).to('cpu',
                                                                          non_blocking=True)
        return res

    # the same with whole-batch copies on the compute stream (no overlap)
    def step_e2e_serial():
        th = theta_h.to(device, non_blocking=True).requires_grad_(True)
        dd = data_h.to(device, non_blocking=True).requires_grad_(True)
        tg = target_h.to(device, non_blocking=True)
        out = T.transform_data(dd, th, [SIZE, SIZE])
        loss = F.mse_loss(out, tg)
        loss.backward()
        res = torch.cat([loss.detach().reshape(1), th.grad.reshape(-1)]).to('cpu',
                                                                          non_blocking=True)
        return res
    for _ in range(2):
        r_pipe = step_e2e()
        r_serial = step_e2e_serial()
    torch.cuda.synchronize()
    e2e_matches = bool(torch.equal(r_pipe, r_serial))
    e2e_times = time_events(step_e2e, args.steps, flush)
    e2e_serial_times = time_events(step_e2e_serial, args.steps, flush)
    barrier()
    ms_e2e = sum(e2e_times) / len(e2e_times)
    ms_e2e_serial = sum(e2e_serial_times) / len(e2e_serial_times)
    h2d = (theta_h.numel() + data_h.numel() + target_h.numel()) * 4
    d2h = (1 + theta_h.numel()) * 4

    # per-kernel timing of the two hot launches (same inputs), for the roofline
    params = T.params
    basis = basis_on(params, device)
    A, _, E = N.cell_tables(NC, NSTEPS, theta, basis)
    lin = torch.cat([torch.linspace(0, 1, SIZE, device=device)] * 2).contiguous()
    out, grid = N.transform_data(NC, NSTEPS, lin, [SIZE, SIZE], E, data, save_grid=True)
    gout = (2.0 / out.numel()) * (out - target)
    ws_need = max(N.load().cpab_transform_data_backward_workspace(
        2, N._ints(NC), NSTEPS, m, N._ints([SIZE, SIZE]), args.batch) for m in (0, 1, 2))
    ws = torch.empty(ws_need, dtype=torch.uint8, device=device)
    # NVTX range "kernel_timing" around the per-kernel timing (launched from
    # this thread; autograd launches the step's backward from its own): a
    # profiler can select these launches (ncu --nvtx --nvtx-include kernel_timing/)
    torch.cuda.nvtx.range_push('kernel_timing')
    t_fwd = time_events(lambda: N.transform_data(NC, NSTEPS, lin, [SIZE, SIZE], E, data,
                                                 save_grid=True), args.steps, flush)
    t_bwd = time_events(lambda: N.transform_data_backward(NC, NSTEPS, 0, lin, [SIZE, SIZE], A, E,
                                                          grid, data, basis, gout,
                                                          workspace=ws), args.steps, flush)
    torch.cuda.nvtx.range_pop()
    # the other gradient modes' fused backward on the same inputs
    t_bwd_modes = {name: time_events(
        lambda m=m: N.transform_data_backward(NC, NSTEPS, m, lin, [SIZE, SIZE], A, E, grid, data,
                                              basis, gout, workspace=ws), args.steps, flush)
        for name, m in (('reference_map', 2), ('exact', 1))}
    # the plain one-kernel-per-op GPU path through the same public API:
    # uniform_meshgrid -> transform_grid -> interpolate (libcpab/cpab.py:304-331
    # unfused), with the same loss and gradients
    mesh = T.uniform_meshgrid([SIZE, SIZE])

    def step_unfused():
        th = theta.detach().requires_grad_(True)
        dd = data.detach().requires_grad_(True)
        out = T.interpolate(dd, T.transform_grid(mesh, th), [SIZE, SIZE])
        loss = F.mse_loss(out, target)
        loss.backward()
        return loss
    for _ in range(2):
        step_unfused()
    t_unf = time_events(step_unfused, args.steps, flush)
    extra = rank == 0 and not args.no_extra
    ragged = run_ragged(device, args.steps, flush, tune=not args.no_tune) if extra else None
    volume = run_volume(device, args.steps, flush, tune=not args.no_tune) if extra else None
    interp = run_interp_sweep(device, args.steps, flush) if extra else None
    aligner = run_aligner(device) if extra else None
    exact = run_exact_flow(device, args.steps, flush) if extra else None
    cfg1 = run_cfg1(device, args.steps, flush) if extra else None
    cfg5 = run_cfg5(device, args.steps, flush) if extra else None
    points = run_ragged_points(device, args.steps, flush, tune=not args.no_tune) if extra else None
    mixed = run_mixed_images(device, args.steps, flush) if extra else None
    # results of the timed inputs on the first images, for the check against
    # the FP64 oracle and the reference's gradient (run on the host after
    # the GPU work): traced trajectories, warped images, dtheta, d(data)
    check = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        n = max(1, min(args.cpu_sample_images, args.batch))
        out_t, cells_t = N.integrate_trace(NC, NSTEPS, mesh, E[:n].contiguous())
        check = {'out': out_t.cpu().numpy(), 'cells': cells_t.cpu().numpy(),
                 'image': out[:n].cpu().numpy(), 'dtheta': e_dth[:n].cpu().numpy(),
                 'ddata': e_dd[:n].cpu().numpy(), 'inputs': (theta_h, data_h, target_h)}
    # the reference's own GPU path on the same inputs (the metric's "plain
    # GPU"), last: it runs code that is not this library's
    plain = None
    if rank == 0 and not args.no_plain:
        plain = run_plain_gpu_reference(device, theta, data, target, flush)
        if extra and 'unavailable' not in plain:
            tg = run_plain_transform_grid(device, flush)
            if cfg1 and 'cfg1_forward_ms' in tg:
                tg['cfg1_forward_speedup'] = tg['cfg1_forward_ms'] / cfg1['forward_ms']
            if cfg5 and 'cfg5_forward_ms' in tg:
                tg['cfg5_forward_speedup'] = tg['cfg5_forward_ms'] / cfg5['forward_ms']
            plain['transform_grid_forward'] = tg
        if '_result' in plain:
            p_loss, p_dth, p_dd, p_grid, p_out = plain.pop('_result')
            # this library's fused backward fed the reference's own warped grid
            # and output (its fp32 step maps T put points up to ~1e-5 from this
            # library's, across bilinear pixel knots where the interpolation
            # gradient jumps): what is left is the gradient arithmetic
            try:
                # the fused kernels keep the grid in output order (last axis
                # fastest); transform_grid returns it in meshgrid order (x fastest)
                nb = p_grid.shape[0]
                p_grid = p_grid.view(nb, 2, SIZE, SIZE).transpose(2, 3).contiguous() \
                    .view(nb, 2, SIZE * SIZE)
                p_gout = (2.0 / p_out.numel()) * (p_out - target)
                o_dd, o_dth = N.transform_data_backward(NC, NSTEPS, 0, lin, [SIZE, SIZE], A, E,
                                                        p_grid, data, basis, p_gout,
                                                        workspace=ws)
                plain['dtheta_rel_diff_on_reference_grid'] = float(
                    (p_dth - o_dth).abs().max() / p_dth.abs().max())
                plain['ddata_rel_diff_on_reference_grid'] = float(
                    (p_dd - o_dd).abs().max() / p_dd.abs().max())
                plain['grid_max_abs_diff_vs_this_library'] = float((p_grid - grid).abs().max())
            except Exception as e:    # report, do not fail the bench
                plain['decomposition_error'] = '%s: %s' % (type(e).__name__, str(e)[:200])
            plain['eager_fused_speedup'] = plain['ms_per_step'] / ms_eager
            plain['headline_speedup'] = plain['ms_per_step'] / ms_step
            plain['target_speedup'] = 5.0
            plain['dtheta_rel_diff_vs_this_library'] = float(
                (p_dth - e_dth).abs().max() / e_dth.abs().max())
            plain['ddata_rel_diff_vs_this_library'] = float(
                (p_dd - e_dd).abs().max() / e_dd.abs().max())
            e_l = e_loss.detach()
            plain['loss_rel_diff_vs_this_library'] = float(abs(p_loss - e_l) / abs(e_l))
            del p_loss, p_dth, p_dd, p_grid, p_out
        torch.cuda.empty_cache()
    clk = clocks.stop() if clocks else None
    status = N.device_status()

    ms_max, ms_e2e_max = reduce_max([ms_step, ms_e2e], device)
    pts = args.batch * SIZE * SIZE
    value = world * pts / (ms_max / 1e3)
    e2e_value = world * pts / (ms_e2e_max / 1e3)

    bwd_ms = sum(t_bwd) / len(t_bwd)
    fwd_ms = sum(t_fwd) / len(t_fwd)
    bwd_flop = pts * NSTEPS * (FLOP_FWD_STEP + FLOP_ADJ_STEP)
    sm_mhz = clk['sm_mhz'] if clk else 2070.0
    sm_max = clk['sm_max_mhz'] if clk and clk.get('sm_max_mhz') else 2070.0
    n_sm = torch.cuda.get_device_properties(device).multi_processor_count
    fp32_peak = n_sm * 128 * 2 * sm_max * 1e6 / 1e12   # TFLOP/s at the maximum SM clock
    issue_peak = n_sm * 4 * sm_mhz * 1e6                # warp instructions/s at the sampled clock
    achieved = bwd_flop / (bwd_ms / 1e3) / 1e12
    fwd_bytes = pts * 8 * CHANNELS
    result = None
    if rank == 0:
        result = {
            'metric': METRIC, 'value': value, 'unit': 'points/s', 'n_gpus': world,
            'steps': args.steps, 'warmup': args.warmup, 'ms_per_step': ms_max,
            'higher_is_better': True, 'scaling': 'weak', 'vs_baseline': None,
            'dtype': 'f32', 'data': 'synthetic',
            'config': {**workload_config(args.batch),
                       'l2': 'flushed before every timed iteration (%d MB write)'
                             % (2 * L2_BYTES // 2 ** 20),
                       'parallelism': 'dp%d' % world,
                       'step': 'public API (transform_data, F.mse_loss, backward) captured in '
                               'one CUDA graph and replayed; eager %.3f ms/step; graph replay '
                               'reproduces the eager dtheta and loss: %s' % (ms_eager,
                                                                              graph_matches)},
            'e2e': {'value': e2e_value, 'unit': 'points/s', 'h2d_bytes_per_step': h2d,
                    'd2h_bytes_per_step': d2h, 'ms_per_step': ms_e2e_max,
                    'path': 'Cpab.transform_data_from_host (images copied on a side stream '
                            'while the trajectories are integrated, then sampled), target '
                            'copied on the same side stream, F.mse_loss, backward, loss + '
                            'dtheta read back; eager',
                    'serial_copies_ms_per_step': ms_e2e_serial,
                    'same_result_as_serial': e2e_matches},
            'gpu_launches': 4 * args.steps,
            'roofline': {'bound': 'fp32', 'kernel': 'k_transform_data_backward (+finalize)',
                         'achieved': achieved, 'peak': fp32_peak, 'unit': 'TFLOP/s',
                         'frac': achieved / fp32_peak,
                         'peak_source': 'derived: %d SMs x 128 FP32 lanes x 2 flop x %.0f MHz '
                                        '(MEASURED_PEAKS has HBM and bf16 only)'
                                        % (n_sm, sm_max),
                         'flop_per_launch': bwd_flop, 'ms_per_launch': bwd_ms,
                         'traffic': BWD_DRAM_BYTES_PER_IMAGE * args.batch,
                         'traffic_unit': 'bytes per launch (ncu dram read+write, 16-image '
                                         'capture scaled by images)'},
            'issue_roofline': {
                'kernel': 'k_transform_data_backward (+finalize)',
                'bound': 'instruction issue (the lookups and the adjoint are branchy scalar '
                         'FP32/integer work, not FMA streams)',
                'warp_instr_per_launch': pts * NSTEPS * INSTR_BWD_STEP / 32,
                'achieved': pts * NSTEPS * INSTR_BWD_STEP / 32 / (bwd_ms / 1e3),
                'peak': issue_peak,
                'unit': 'warp instructions/s',
                'frac': pts * NSTEPS * INSTR_BWD_STEP / 32 / (bwd_ms / 1e3) / issue_peak,
                'forward_frac': pts * NSTEPS * INSTR_FWD_STEP / 32 / (fwd_ms / 1e3) / issue_peak,
                'source': 'instructions per point-step from ncu (%d bwd, %d fwd); peak = '
                          '%d SMs x 4 schedulers x 1 instruction/cycle at the sampled SM '
                          'clock' % (INSTR_BWD_STEP, INSTR_FWD_STEP, n_sm)},
            'launch_shapes': shapes,
            'backward_ms_per_launch_by_gradient_mode': {
                'reference': bwd_ms,
                **{k: sum(v) / len(v) for k, v in t_bwd_modes.items()},
                'note': "k_transform_data_backward + k_finalize; 'reference' (the default and "
                        "the headline) follows the reference's midpoint trajectory in its own "
                        "arithmetic, 'reference_map' the collapsed per-cell midpoint map, "
                        "'exact' is the exact adjoint of the forward map"},
            'forward_kernel': {'name': 'k_transform_data', 'ms_per_launch': fwd_ms,
                               'flop_per_launch': pts * NSTEPS * FLOP_FWD_STEP,
                               'tflops': pts * NSTEPS * FLOP_FWD_STEP / (fwd_ms / 1e3) / 1e12,
                               'interp_gbs': fwd_bytes / (fwd_ms / 1e3) / 1e9},
            'unfused_gpu': {'path': 'transform_grid -> interpolate -> MSE, autograd '
                                    '(cpab_integrate, cpab_interpolate and their backward '
                                    'kernels, one launch per op)',
                            'ms_per_step': sum(t_unf) / len(t_unf),
                            'value': pts / (sum(t_unf) / len(t_unf) / 1e3),
                            'unit': 'points/s'},
            'plain_gpu_reference': plain,
            'ragged_1d': ragged,
            'volume_3d': volume,
            'interpolate_2d': interp,
            'aligner': aligner,
            'exact_flow': exact,
            'cfg1_transform_grid_1d': cfg1,
            'cfg5_precision_stress_2d': cfg5,
            'ragged_points_2d': points,
            'mixed_size_images_2d': mixed,
            'clocks': clk, 'device_status': status,
            '_check': check,
        }
    if world > 1:
        torch.distributed.destroy_process_group()
    return result


def tune_headline(T, theta, data, device, flush, steps=10):
    """The fused forward's and backward's per-launch times with the built-in
    launch heuristics, then the autotuner on the same inputs (reference
    gradient), then the times with the kept shapes.  Shapes are (threads per
    CTA, points per thread, CTAs per image, per-warp table staging)."""
    from libcpab_gb300 import _native as N
    from libcpab_gb300.functions import basis_on, grid_axes
    basis = basis_on(T.params, device)
    A, _, E = N.cell_tables(NC, NSTEPS, theta, basis)
    lin = grid_axes(T.params, [SIZE, SIZE], device)
    out, grid = N.transform_data(NC, NSTEPS, lin, [SIZE, SIZE], E, data, save_grid=True)
    gout = torch.randn(out.shape, generator=torch.Generator().manual_seed(9)).to(device)
    fwd = lambda: N.transform_data(NC, NSTEPS, lin, [SIZE, SIZE], E, data, save_grid=True)
    bwd = lambda: N.transform_data_backward(NC, NSTEPS, 0, lin, [SIZE, SIZE], A, E, grid, data,
                                            basis, gout)

    def times():
        for _ in range(3):
            fwd()
            bwd()
        tf, tb = time_events(fwd, steps, flush), time_events(bwd, steps, flush)
        return sum(tf) / len(tf), sum(tb) / len(tb)
    f0, b0 = times()
    res = T.tune_transform_data(data, theta, [SIZE, SIZE])
    f1, b1 = times()
    return {'forward': {'kernel': 'k_transform_data', 'shape': list(res['forward'][0]),
                        'ms_heuristic': f0, 'ms_tuned': f1},
            'backward': {'kernel': 'k_transform_data_backward (+finalize)',
                         'shape': list(res['backward'][0]), 'ms_heuristic': b0, 'ms_tuned': b1},
            'fields': 'threads per CTA, points per thread, CTAs per image, per-warp tables '
                      '(0 shared, 1 global memory)'}


# ragged batched 1D series: 4,096 series, lengths U{32..4096}, tess [100]
RAGGED_S, RAGGED_NC, RAGGED_LEN = 4096, 100, (32, 4096)


def ragged_inputs(T, device):
    """Series values = sum of 3 sinusoids (f ~ U[1,10], phase ~ U[0,2pi],
    amplitude ~ U[0.5,1.5]) + N(0, 0.1^2) on linspace(0, 1, L_s); theta ~ N(0, I)
    (seed 0), data (seed 1), target = the values warped by a second theta
    (seed 2)."""
    from libcpab_gb300 import _native as N
    from libcpab_gb300.functions import basis_on
    d = T.get_theta_dim()
    g0, g1, g2 = (torch.Generator().manual_seed(k) for k in (0, 1, 2))
    theta = torch.randn(RAGGED_S, d, generator=g0)
    lengths = torch.randint(RAGGED_LEN[0], RAGGED_LEN[1] + 1, (RAGGED_S,), generator=g1)
    off = torch.cat([torch.zeros(1, dtype=torch.int64), torch.cumsum(lengths, 0)])
    sid = torch.repeat_interleave(torch.arange(RAGGED_S), lengths)
    j = torch.arange(int(off[-1])) - off[sid]
    x = j.double() / (lengths[sid] - 1).double()
    f = 1 + 9 * torch.rand(RAGGED_S, 3, generator=g1, dtype=torch.float64)
    ph = 2 * np.pi * torch.rand(RAGGED_S, 3, generator=g1, dtype=torch.float64)
    amp = 0.5 + torch.rand(RAGGED_S, 3, generator=g1, dtype=torch.float64)
    v = (amp[sid] * torch.sin(2 * np.pi * f[sid] * x[:, None] + ph[sid])).sum(1)
    v = v + 0.1 * torch.randn(v.shape, generator=g1, dtype=torch.float64)
    values = v.float().to(device)
    off = off.to(device)
    theta2 = torch.randn(RAGGED_S, d, generator=g2).to(device)
    basis = basis_on(T.params, device)
    _, _, E2 = N.cell_tables([RAGGED_NC], NSTEPS, theta2, basis)
    target = N.ragged_forward([RAGGED_NC], NSTEPS, E2, off, values)
    return theta.to(device), off, values, target, basis


def run_ragged(device, steps, flush, tune=True):
    """Fused forward + MSE + dtheta/d(values) adjoint of the ragged workload in
    one persistent launch (plus the tile-prefix and finalize kernels and the
    cell tables), autotuned, captured in a CUDA graph and replayed."""
    from libcpab_gb300 import Cpab, _native as N
    T = Cpab([RAGGED_NC], backend='pytorch', device='gpu', zero_boundary=False)
    theta, off, values, target, basis = ragged_inputs(T, device)
    total = values.numel()
    A, _, E = N.cell_tables([RAGGED_NC], NSTEPS, theta, basis)
    ws = N.ragged_workspace(RAGGED_NC, NSTEPS, RAGGED_S, device)
    shape_f = shape_b = ms_f = None
    if tune:
        shape_f, ms_f, _ = N.ragged_tune(0, [RAGGED_NC], NSTEPS, 0, A, E, off, values, target,
                                         basis, workspace=ws)
        shape_b, _, _ = N.ragged_tune(1, [RAGGED_NC], NSTEPS, 0, A, E, off, values, target,
                                      basis, workspace=ws)
    st = torch.cuda.Stream()
    st.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(st):
        for _ in range(3):
            A, _, E = N.cell_tables([RAGGED_NC], NSTEPS, theta, basis)
            N.ragged_mse([RAGGED_NC], NSTEPS, 0, A, E, off, values, target, basis, workspace=ws)
    torch.cuda.current_stream().wait_stream(st)
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        A, _, E = N.cell_tables([RAGGED_NC], NSTEPS, theta, basis)
        res = N.ragged_mse([RAGGED_NC], NSTEPS, 0, A, E, off, values, target, basis,
                           workspace=ws)
    for _ in range(3):
        g.replay()
    times = time_events(g.replay, steps, flush)
    ms = sum(times) / len(times)
    loss = float(res['sse'].sum()) / total
    return {'workload': 'ragged 1D: %d series, lengths U{%d..%d} (total %d points), tess [%d] '
                        'zero_boundary=False, theta ~ N(0,I), sum-of-sinusoids values, MSE vs '
                        'values warped by a second theta, fwd + dtheta/d(values) (reference '
                        'gradient) in one persistent launch, CUDA-graph replay'
                        % (RAGGED_S, RAGGED_LEN[0], RAGGED_LEN[1], total, RAGGED_NC),
            'value': total / (ms / 1e3), 'unit': 'points/s', 'ms_per_step': ms,
            'launches_per_step': 4, 'tuned_shape_fused': list(shape_b) if shape_b else None,
            'tuned_shape_forward': list(shape_f) if shape_f else None,
            'forward_only_ms': ms_f,
            'loss': loss}


POINTS_S, POINTS_LEN = 1024, (256, 16384)


def run_ragged_points(device, steps, flush, tune=True):
    """Ragged point sets in 2D (tess [3,3] zero_boundary, the headline
    tessellation): 1,024 sets of U{256..16384} points ~ U[0,1]^2, theta ~
    N(0, 0.25 I) per set.  Forward alone and forward + dtheta backward
    (reference gradient) in one persistent launch each, on the points as given
    and on the points sorted by starting cell; beside them the padded
    alternative (one batched transform_grid call on sets padded to the
    longest)."""
    from libcpab_gb300 import Cpab, _native as N
    from libcpab_gb300.functions import basis_on, findcellidx
    T = Cpab(NC, backend='pytorch', device='gpu', zero_boundary=True)
    g = torch.Generator().manual_seed(3)
    theta = (THETA_STD * torch.randn(POINTS_S, T.get_theta_dim(), generator=g)).to(device)
    lengths = torch.randint(POINTS_LEN[0], POINTS_LEN[1] + 1, (POINTS_S,), generator=g)
    off = torch.cat([torch.zeros(1, dtype=torch.int64), torch.cumsum(lengths, 0)]).to(device)
    total = int(lengths.sum())
    pts = torch.rand(2, total, generator=g).to(device)
    basis = basis_on(T.params, device)
    A, _, E = N.cell_tables(NC, NSTEPS, theta, basis)
    gout = torch.randn(2, total, generator=g).to(device)
    nC = N.num_cells(NC)
    pos = torch.arange(total, device=device)
    sid = torch.searchsorted(off, pos, right=True) - 1
    perm = torch.sort(sid * nC + findcellidx(2, pts, NC), stable=True).indices
    pts_sorted, gout_sorted = pts[:, perm].contiguous(), gout[:, perm].contiguous()
    wsf = N.ragged_points_workspace(NC, POINTS_S, device)
    wsb = N.ragged_points_workspace(NC, POINTS_S, device)
    res = {}
    if tune:
        # tuned on the sorted points (the order sort_by_cell runs); the kept
        # shapes serve both orders (the problem key is the sets' sizes)
        tuned = T.tune_transform_grid_ragged(pts_sorted, off, theta)
        res['launch_shapes'] = {k: list(v[0]) for k, v in tuned.items()}
    for tag, P, G in (('unsorted', pts, gout), ('sorted', pts_sorted, gout_sorted)):
        fwd = lambda: N.ragged_points_forward(NC, NSTEPS, E, off, P, workspace=wsf)
        bwd = lambda: N.ragged_points_backward(NC, NSTEPS, 0, A, E, off, P, basis, G,
                                               workspace=wsb)
        for _ in range(3):
            fwd(); bwd()
        tf = time_events(fwd, steps, flush)
        tb = time_events(bwd, steps, flush)
        ms_f, ms_b = sum(tf) / len(tf), sum(tb) / len(tb)
        res[tag] = {'forward_ms': ms_f, 'backward_ms': ms_b,
                    'forward_points_per_s': total / (ms_f / 1e3),
                    'fwd_bwd_points_per_s': total / ((ms_f + ms_b) / 1e3)}
    # the padded alternative: sets padded to the longest, one batched call
    Lmax = int(lengths.max())
    padded = torch.full((POINTS_S, 2, Lmax), 0.5, device=device)
    for s in range(POINTS_S):
        a, b = int(off[s]), int(off[s + 1])
        padded[s, :, :b - a] = pts[:, a:b]
    gpad = torch.zeros_like(padded)
    for _ in range(2):
        N.integrate(NC, NSTEPS, padded, E)
    tp = time_events(lambda: N.integrate(NC, NSTEPS, padded, E), max(2, steps // 4), flush)
    tpb = time_events(lambda: N.backward(NC, NSTEPS, 0, padded, A, E, basis, gpad),
                      max(2, steps // 4), flush)
    ms_p, ms_pb = sum(tp) / len(tp), sum(tpb) / len(tpb)
    res['padded_batch'] = {'forward_ms': ms_p, 'backward_ms': ms_pb,
                           'fwd_bwd_points_per_s': total / ((ms_p + ms_pb) / 1e3),
                           'padded_points': POINTS_S * Lmax}
    res['workload'] = ('ragged point sets 2D: %d sets of U{%d..%d} points ~ U[0,1]^2 (total %d), '
                       'tess [3,3] zero_boundary, theta ~ N(0,0.25I) per set; forward and '
                       'forward+dtheta (reference gradient), one persistent launch each'
                       % (POINTS_S, POINTS_LEN[0], POINTS_LEN[1], total))
    return res


MIXED_S, MIXED_SIDE = 64, (128, 320)


def run_mixed_images(device, steps, flush):
    """Images of mixed sizes: 64 images [3, W, H] with W, H ~ U{128..320}
    (values U[0,1]), each warped to its own size by its own theta ~
    N(0, 0.25 I), tess [3,3] zero_boundary.  One step = forward + backward
    (reference gradient, dtheta and d(images)) of sum(out_s * w_s) through
    Cpab.transform_data_mixed (one ragged integration launch, one ragged
    sampling launch, and their adjoints); beside it the same step as a loop of
    per-image transform_data calls (what the reference's API allows), and the
    mixed step captured in a CUDA graph and replayed."""
    from libcpab_gb300 import Cpab
    T = Cpab(NC, backend='pytorch', device='gpu', zero_boundary=True)
    T.set_solver_params(nstepsolver=NSTEPS)
    g = torch.Generator().manual_seed(5)
    sides = torch.randint(MIXED_SIDE[0], MIXED_SIDE[1] + 1, (MIXED_S, 2), generator=g).tolist()
    ims = [torch.rand(CHANNELS, w, h, generator=g).to(device) for w, h in sides]
    ws = [torch.randn(CHANNELS, w, h, generator=g).to(device) for w, h in sides]
    theta = (THETA_STD * torch.randn(MIXED_S, T.get_theta_dim(), generator=g)).to(device)
    total = sum(w * h for w, h in sides)

    def step_mixed():
        th = theta.detach().requires_grad_(True)
        dd = [im.detach().requires_grad_(True) for im in ims]
        torch.autograd.backward(T.transform_data_mixed(dd, th), ws)
        return th.grad

    def step_loop():
        th = theta.detach().requires_grad_(True)
        for s in range(MIXED_S):
            d = ims[s][None].detach().requires_grad_(True)
            torch.autograd.backward(T.transform_data(d, th[s:s + 1], sides[s]), ws[s][None])
        return th.grad

    res = {}
    for tag, fn in (('mixed', step_mixed), ('per_image_loop', step_loop)):
        for _ in range(3):
            fn()
        t = time_events(fn, steps, flush)
        ms = sum(t) / len(t)
        res[tag] = {'ms_per_step': ms, 'fwd_bwd_points_per_s': total / (ms / 1e3)}
    a, b = step_mixed(), step_loop()
    res['dtheta_rel_diff'] = float((a - b).abs().max() / b.abs().max())
    # the mixed step captured once in a CUDA graph and replayed (the layout
    # is cached by the eager calls above, so the capture only records kernels)
    side = torch.cuda.Stream()
    side.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(side):
        for _ in range(2):
            step_mixed()
    torch.cuda.current_stream().wait_stream(side)
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph):
        g_dth = step_mixed()
    for _ in range(3):
        graph.replay()
    t = time_events(graph.replay, steps, flush)
    ms = sum(t) / len(t)
    res['mixed_graph'] = {'ms_per_step': ms, 'fwd_bwd_points_per_s': total / (ms / 1e3),
                          'dtheta_equals_eager': bool(torch.equal(g_dth, a))}
    res['workload'] = ('images of mixed sizes: %d images [%d, W, H], W, H ~ U{%d..%d} (total %d '
                       'points), each warped to its size by its own theta ~ N(0,0.25I), tess '
                       '[3,3] zero_boundary; forward + backward (dtheta, d(images)) of '
                       'sum(out * w)' % (MIXED_S, CHANNELS, MIXED_SIDE[0], MIXED_SIDE[1], total))
    return res


PLAIN_STEPS = 3


def run_plain_gpu_reference(device, theta, data, target, flush, steps=PLAIN_STEPS):
    """The headline step through the reference's own pytorch GPU path, run
    unmodified from baseline/_ref (baseline/plain_gpu.py): Cpab.transform_data
    (basis upload, Pade expm with its host sync, the cpab_gpu forward kernel,
    gather interpolation), F.mse_loss and autograd (the cpab_gpu analytic
    backward writing the [d, n_theta, 2, nP] sensitivity tensor, its
    contraction, the interpolation's scatter backward).  Same inputs, eager,
    L2 flushed before each timed step.  Returns a dict, or one with
    'unavailable' when the reference op is not built."""
    try:
        from baseline import plain_gpu
        from libcpab_gb300.tessellation import make_tessellation
        ref = plain_gpu.load()
        # override: the reference builds its basis here, with this machine's
        # LAPACK, as this library does (a null-space basis from an SVD is
        # only defined up to rotation, so a basis file from another machine
        # would give theta another meaning)
        T = ref.Cpab(NC, backend='pytorch', device='gpu', zero_boundary=True, override=True)
        basis_diff = float(np.abs(T.params.basis - make_tessellation(NC, True, False).B).max())

        def step():
            th = theta.detach().requires_grad_(True)
            dd = data.detach().requires_grad_(True)
            out = T.transform_data(dd, th, [SIZE, SIZE])
            loss = F.mse_loss(out, target)
            loss.backward()
            return loss.detach(), th.grad, dd.grad
        loss, dth, dd = step()
        with torch.no_grad():   # its warped grid and output, for the decomposition
            mesh = T.uniform_meshgrid([SIZE, SIZE])
            ref_grid = T.transform_grid(mesh, theta).contiguous()
            ref_out = T.interpolate(data, ref_grid, [SIZE, SIZE]).contiguous()
        torch.cuda.synchronize()
        t = time_events(step, steps, flush)
    except Exception as e:    # the comparator is optional: report, do not fail the bench
        return {'unavailable': '%s: %s' % (type(e).__name__, str(e)[:300])}
    ms = statistics.median(t)
    pts = theta.shape[0] * SIZE * SIZE
    return {'path': "reference libcpab, unmodified (baseline/_ref): Cpab.transform_data "
                    "(backend='pytorch', device='gpu') + F.mse_loss + backward; its CUDA op "
                    "JIT-built for sm_103a by its own torch.utils.cpp_extension.load",
            'ms_per_step': ms, 'ms_all': t, 'value': pts / (ms / 1e3), 'unit': 'points/s',
            'steps': steps, 'chunking': 'none: its [34, 64, 2, 50176] sensitivity tensor '
                                        '(873 MB) fits',
            'basis_max_abs_diff_vs_this_library': basis_diff,
            '_result': (loss, dth, dd, ref_grid, ref_out)}


def run_plain_transform_grid(device, flush, steps=3):
    """The reference's own GPU transform_grid (forward: its basis upload, Pade
    expm and cpab_gpu forward kernel) on the cfg1 and cfg5 inputs of
    run_cfg1 / run_cfg5 (same seeds), for the forward ratio beside the
    headline's.  The reference builds its basis on this machine (override)."""
    try:
        from baseline import plain_gpu
        ref = plain_gpu.load()
        res = {}
        # cfg1: tess [50] zero boundary, 16 theta ~ N(0, I), 1,000-point meshgrid
        T1 = ref.Cpab([50], backend='pytorch', device='gpu', zero_boundary=True, override=True)
        th1 = torch.randn(16, T1.get_theta_dim(),
                          generator=torch.Generator().manual_seed(0)).to(device)
        g1 = T1.uniform_meshgrid([1000])
        for _ in range(3):
            T1.transform_grid(g1, th1)
        t = time_events(lambda: T1.transform_grid(g1, th1), max(steps, 10), flush)
        res['cfg1_forward_ms'] = statistics.median(t)
        # cfg5: tess [8,8] free, 256 theta ~ N(0, 9 I) + 256 ~ 1e-6 N(0, I), 512^2 grid
        T5 = ref.Cpab([8, 8], backend='pytorch', device='gpu', zero_boundary=False,
                      override=True)
        d = T5.get_theta_dim()
        g = torch.Generator().manual_seed(0)
        th5 = torch.cat([3.0 * torch.randn(256, d, generator=g),
                         1e-6 * torch.randn(256, d, generator=g)]).to(device)
        lin = torch.linspace(0, 1, 512)
        gx, gy = torch.meshgrid(lin, lin, indexing='xy')
        g5 = torch.stack([gx.reshape(-1), gy.reshape(-1)]).contiguous().to(device)
        T5.transform_grid(g5, th5[:16])
        t = time_events(lambda: T5.transform_grid(g5, th5), max(1, steps), flush)
        res['cfg5_forward_ms'] = statistics.median(t)
        res['path'] = ("reference libcpab, unmodified: Cpab.transform_grid (backend='pytorch', "
                       "device='gpu'), forward only, all theta in one call")
        return res
    except Exception as e:    # the comparator is optional: report, do not fail the bench
        return {'unavailable': '%s: %s' % (type(e).__name__, str(e)[:300])}


def run_plain_leg(device, steps, flush):
    """The plain comparator alone on the headline inputs (for profiling runs)."""
    from libcpab_gb300 import Cpab
    T = Cpab(NC, backend='pytorch', device='gpu', zero_boundary=True)
    theta, data, target = make_inputs(T, device)
    res = run_plain_gpu_reference(device, theta.to(device), data.to(device),
                                  target.to(device), flush, steps=max(1, steps))
    res.pop('_result', None)
    return res


def hbm_peak():
    """Measured copy bandwidth of this GPU model (GB/s), else the fallback."""
    try:
        with open(os.path.join(HERE, 'MEASURED_PEAKS.json')) as f:
            return float(json.load(f)['hbm_gbs']), 'measured (MEASURED_PEAKS.json hbm_gbs)'
    except (OSError, ValueError, KeyError):
        return 6800.0, 'fallback'


def make_volumes(device, nb=8, size=128, blobs=32, seed=1):
    """[nb, 1, size^3] volumes, each a sum of `blobs` isotropic Gaussian blobs
    (centres uniform in the volume, sigma ~ U[2, 8] voxels, amplitude ~
    U[0.5, 1])."""
    g = torch.Generator().manual_seed(seed)
    centres = (torch.rand(nb, blobs, 3, generator=g) * size).to(device)
    sigma = (2 + 6 * torch.rand(nb, blobs, generator=g)).to(device)
    amp = (0.5 + 0.5 * torch.rand(nb, blobs, generator=g)).to(device)
    ax = torch.arange(size, dtype=torch.float32, device=device)
    f = torch.exp(-(ax[None, None, None, :] - centres[..., None]) ** 2
                  / (2 * sigma[..., None, None] ** 2))               # [nb, blobs, 3, size]
    vol = torch.einsum('nb,nbx,nby,nbz->nxyz', amp, f[:, :, 0], f[:, :, 1], f[:, :, 2])
    return vol[:, None].contiguous()


def run_volume(device, steps, flush, tune=True):
    """3D volume warp: tess [4,4,4] zero_boundary + volume_perservation, 8 theta
    ~ N(0, I), [8, 1, 128^3] blob volumes, MSE against the volumes warped by a
    second theta; fused forward + dtheta/d(data) backward through the public
    API.  Also the trilinear interpolator alone (HBM-bound)."""
    from libcpab_gb300 import Cpab, _native as N
    T = Cpab([4, 4, 4], backend='pytorch', device='gpu', zero_boundary=True,
             volume_perservation=True)
    d = T.get_theta_dim()
    theta = torch.randn(8, d, generator=torch.Generator().manual_seed(0)).to(device)
    theta2 = torch.randn(8, d, generator=torch.Generator().manual_seed(2)).to(device)
    data = make_volumes(device)
    osz = [128, 128, 128]
    with torch.no_grad():
        target = T.transform_data(data, theta2, osz)

    def step():
        th = theta.detach().requires_grad_(True)
        dd = data.detach().requires_grad_(True)
        loss = F.mse_loss(T.transform_data(dd, th, osz), target)
        loss.backward()
        return loss
    for _ in range(3):
        step()
    shapes = None
    if tune:
        t_heur = time_events(step, steps, flush)
        tuned = T.tune_transform_data(data, theta, osz)
        for _ in range(2):
            step()
        shapes = {'forward': list(tuned['forward'][0]), 'backward': list(tuned['backward'][0]),
                  'ms_per_step_heuristic': sum(t_heur) / len(t_heur)}
    t_step = time_events(step, steps, flush)
    grid = T.transform_grid(T.uniform_meshgrid(osz), theta)
    for _ in range(3):
        N.interpolate(data, grid, osz)
    t_int = time_events(lambda: N.interpolate(data, grid, osz), steps, flush)
    pts = 8 * 128 ** 3
    ms, ms_i = sum(t_step) / len(t_step), sum(t_int) / len(t_int)
    peak, src = hbm_peak()
    gbs = pts * 20 / (ms_i / 1e3) / 1e9     # data read + output write 8 B (C = 1), grid 12 B
    return {'workload': 'transform_data 3D tess [4,4,4] zero_boundary volume_perservation, 8 '
                        'theta ~ N(0,I), [8,1,128^3] Gaussian-blob volumes, MSE, fwd + '
                        'dtheta/d(data) bwd (reference gradient)',
            'value': pts / (ms / 1e3), 'unit': 'points/s', 'ms_per_step': ms,
            'launch_shapes': shapes,
            'interpolate': {'ms': ms_i, 'algorithmic_bytes': pts * 20, 'gbs': gbs,
                            'frac_of_hbm': gbs / peak, 'peak_gbs': peak, 'peak_source': src}}


def run_interp_sweep(device, steps, flush):
    """Bilinear interpolator alone (cpab_interpolate) on [nb, 3, 224, 224] with
    CPAB-warped grids (tess [3,3], theta ~ N(0, 0.25 I)).  Algorithmic bytes
    per output point: 8 C (data read once, output written once) + 4 ndim (the
    grid, an input of the standalone op), against the measured HBM
    bandwidth."""
    from libcpab_gb300 import Cpab, _native as N
    peak, src = hbm_peak()
    T = Cpab(NC, backend='pytorch', device='gpu', zero_boundary=True)
    mesh = T.uniform_meshgrid([SIZE, SIZE])
    res = []
    for nb in (64, 256, 1024):
        g = torch.Generator(device=device).manual_seed(nb)
        data = torch.rand(nb, 3, SIZE, SIZE, device=device, generator=g)
        th = THETA_STD * torch.randn(nb, T.get_theta_dim(), device=device, generator=g)
        with torch.no_grad():
            grid = T.transform_grid(mesh, th)
        for _ in range(3):
            N.interpolate(data, grid, [SIZE, SIZE])
        t = time_events(lambda: N.interpolate(data, grid, [SIZE, SIZE]), steps, flush)
        ms = sum(t) / len(t)
        nbytes = nb * SIZE * SIZE * (8 * 3 + 4 * 2)
        gbs = nbytes / (ms / 1e3) / 1e9
        res.append({'n_batch': nb, 'ms': ms, 'algorithmic_bytes': nbytes, 'gbs': gbs,
                    'frac_of_hbm': gbs / peak})
        del data, grid
    return {'sweep': res, 'peak_gbs': peak, 'peak_source': src}


def run_aligner(device, iters=100):
    """CpabAligner.alignment_by_gradient on one 3 x 224 x 224 image (tess [3,3],
    Adam, lr 1e-2): the eager loop (losses kept on the device) against the
    same loop replayed from a CUDA graph."""
    from libcpab_gb300 import Cpab, CpabAligner
    T = Cpab(NC, backend='pytorch', device='gpu', zero_boundary=True)
    g = torch.Generator().manual_seed(4)
    raw = torch.rand(1, CHANNELS, SIZE, SIZE, generator=g)
    x1 = F.avg_pool2d(raw, 5, 1, 2, count_include_pad=False).to(device).contiguous()
    th_true = (THETA_STD * torch.randn(1, T.get_theta_dim(), generator=g)).to(device)
    with torch.no_grad():
        x2 = T.transform_data(x1, th_true, [SIZE, SIZE])
    A = CpabAligner(T)
    res = {}
    for name, graph in (('eager', False), ('graph', True)):
        A.alignment_by_gradient(x1, x2, maxiter=5, graph=graph)     # warm-up
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        A.alignment_by_gradient(x1, x2, maxiter=iters, graph=graph)
        losses = A.losses.cpu()
        dt = time.perf_counter() - t0
        res[name] = {'iterations_per_s': iters / dt, 'final_loss': float(losses[-1]),
                     'first_loss': float(losses[0])}
    res['workload'] = ('alignment_by_gradient, 1 x 3 x 224^2, tess [3,3], %d Adam iterations '
                       '(wall clock incl. graph capture)' % iters)
    return res


def run_exact_flow(device, steps, flush):
    """The opt-in exact-flow scheme on the headline grid (tess [3,3],
    64 theta ~ N(0, 0.25 I), 224^2 grid): transform_grid forward and its
    dtheta backward (reverse sweep), against the fixed-step scheme on the same
    points."""
    from libcpab_gb300 import Cpab, _native as N
    from libcpab_gb300.functions import basis_on
    T = Cpab(NC, backend='pytorch', device='gpu', zero_boundary=True)
    theta = (THETA_STD * torch.randn(BATCH, T.get_theta_dim(),
                                     generator=torch.Generator().manual_seed(0))).to(device)
    basis = basis_on(T.params, device)
    A, _, E = N.cell_tables(NC, NSTEPS, theta, basis)
    grid = T.uniform_meshgrid([SIZE, SIZE])
    for _ in range(3):
        N.integrate_exact(NC, grid, A)
        N.integrate(NC, NSTEPS, grid, E)
    t_ex = time_events(lambda: N.integrate_exact(NC, grid, A), steps, flush)
    t_fs = time_events(lambda: N.integrate(NC, NSTEPS, grid, E), steps, flush)
    cnt = torch.zeros(1, dtype=torch.int64, device=device)
    ex = N.integrate_exact(NC, grid, A, steps=cnt)
    fs = N.integrate(NC, NSTEPS, grid, E)
    gout = torch.randn(ex.shape, generator=torch.Generator().manual_seed(5)).to(device)
    for _ in range(2):
        N.backward_exact(NC, ex, A, basis, gout)
    t_bw = time_events(lambda: N.backward_exact(NC, ex, A, basis, gout), max(2, steps // 2),
                       flush)
    pts = BATCH * SIZE * SIZE
    ms_ex, ms_fs = sum(t_ex) / len(t_ex), sum(t_fs) / len(t_fs)
    ms_bw = sum(t_bw) / len(t_bw)
    return {'workload': 'transform_grid, tess [3,3] zero_boundary, 64 theta ~ N(0,0.25I), '
                        '224^2 grid',
            'exact_ms': ms_ex, 'exact_points_per_s': pts / (ms_ex / 1e3),
            'exact_backward_ms': ms_bw,
            'fixed_step_ms': ms_fs, 'in_cell_steps_per_point': int(cnt.item()) / pts,
            'max_abs_diff_exact_vs_fixed_step': float((ex - fs).abs().max())}


def trajectory_errors(B, theta, pts, nc, out, cells):
    """GPU trajectories [n, ndim, nP] (with their cells [n, nP, nsteps])
    against the FP64 oracle of the same scheme (C++ cell rules): max and p99
    error of the trajectories with the oracle's cells (scaled by max(1, |p|)),
    and the others (boundary ties) with the margin at their first divergence."""
    from oracle.oracle import numpy_transform_grid
    ref, cells64, marg = numpy_transform_grid(B, theta, pts, nc, NSTEPS, return_cells=True,
                                              return_margin='steps', semantics='cpp')
    diff = cells != cells64
    tie = diff.any(axis=2)
    err = np.abs(out - ref).max(axis=1) / np.maximum(1.0, np.abs(ref).max(axis=1))
    first = diff.argmax(axis=2)
    ti, pi = np.nonzero(tie)
    fm = marg[ti, pi, first[ti, pi]] if ti.size else np.zeros(0)
    clean = err[~tie]
    return {'trajectories': int(err.size),
            'clean_max_err': float(clean.max()) if clean.size else 0.0,
            'clean_p99_err': float(np.quantile(clean, 0.99)) if clean.size else 0.0,
            'tie_trajectories': int(tie.sum()),
            'tie_first_margin_max': float(fm.max()) if fm.size else 0.0}


def run_cfg1(device, steps, flush):
    """The reference's CPU-runnable configuration: tess [50] zero_boundary,
    16 theta ~ N(0, I), transform_grid of the 1,000-point meshgrid.  Forward
    (cell tables + integration) and forward + dtheta backward through the
    public API on the GPU; beside them the reference's own compiled C++ op
    (pytorch-CPU path, its fp32 step maps) and the FP64 restatement of its
    numpy backend on one host core each, and the GPU's error against FP64."""
    from libcpab_gb300 import Cpab, _native as N
    from libcpab_gb300.functions import basis_on
    from oracle.oracle import RefLib, numpy_transform_grid
    nc = [50]
    T = Cpab(nc, backend='pytorch', device='gpu', zero_boundary=True)
    theta = torch.randn(16, T.get_theta_dim(), generator=torch.Generator().manual_seed(0))
    th = theta.to(device)
    grid = T.uniform_meshgrid([1000])
    fwd = lambda: T.transform_grid(grid, th)

    def fwd_bwd():
        t = th.detach().requires_grad_(True)
        T.transform_grid(grid, t).sum().backward()
    for _ in range(5):
        fwd()
        fwd_bwd()
    n = max(steps, 20)
    tf, tb = time_events(fwd, n, flush), time_events(fwd_bwd, n, flush)
    basis = basis_on(T.params, device)
    _, Tt, E = N.cell_tables(nc, NSTEPS, th, basis, want_T=True)
    out, cells = N.integrate_trace(nc, NSTEPS, grid, E)
    B = T.params.basis
    pts = grid.cpu().numpy()
    errs = trajectory_errors(B, theta.numpy(), pts, nc, out.cpu().numpy(), cells.cpu().numpy())
    pts_n = 16 * 1000
    res = {'workload': 'transform_grid, tess [50] zero_boundary, 16 theta ~ N(0,I), 1,000-point '
                       'meshgrid', 'forward_ms': sum(tf) / len(tf),
           'forward_points_per_s': pts_n / (sum(tf) / len(tf) / 1e3),
           'fwd_bwd_ms': sum(tb) / len(tb),
           'fwd_bwd_points_per_s': pts_n / (sum(tb) / len(tb) / 1e3),
           'error_vs_fp64': errs}
    # the reference's CPU paths on the same inputs (one core each)
    try:
        ref = RefLib()
        trels = Tt.cpu().numpy()
        ref.forward(nc, NSTEPS, pts, trels)
        t0 = time.perf_counter()
        reps = 20
        for _ in range(reps):
            ref.forward(nc, NSTEPS, pts, trels)
        ms = (time.perf_counter() - t0) / reps * 1e3
        res['reference_cpp_cpu_forward'] = {'ms': ms, 'points_per_s': pts_n / (ms / 1e3),
                                            'cores': 1}
    except (OSError, FileNotFoundError) as e:
        res['reference_cpp_cpu_forward'] = {'unavailable': str(e)[:200]}
    t0 = time.perf_counter()
    numpy_transform_grid(B, theta.numpy(), pts, nc, NSTEPS)
    ms = (time.perf_counter() - t0) * 1e3
    res['reference_numpy_fp64_forward'] = {'ms': ms, 'points_per_s': pts_n / (ms / 1e3),
                                           'cores': 1,
                                           'path': 'FP64 restatement of the numpy backend'}
    return res


def run_cfg5(device, steps, flush):
    """The precision-stress configuration: tess [8,8] without zero boundary
    (d = 234), 256 theta ~ N(0, 9 I) and 256 theta ~ 1e-6 N(0, I), the 512 x
    512 grid per theta (134 M trajectories): transform_grid forward and its
    dtheta backward (reference gradient) on the GPU, the FP64-path lookups
    over the whole run, and the error against the FP64 oracle on a sample
    (8 theta of each group x 1,024 grid points)."""
    from libcpab_gb300 import Cpab, _native as N
    from libcpab_gb300.functions import basis_on
    nc = [8, 8]
    T = Cpab(nc, backend='pytorch', device='gpu', zero_boundary=False)
    d = T.get_theta_dim()
    g = torch.Generator().manual_seed(0)
    theta = torch.cat([3.0 * torch.randn(256, d, generator=g),
                       1e-6 * torch.randn(256, d, generator=g)])
    th = theta.to(device)
    lin = torch.linspace(0, 1, 512)
    gx, gy = torch.meshgrid(lin, lin, indexing='xy')
    grid = torch.stack([gx.reshape(-1), gy.reshape(-1)]).contiguous()
    P = grid.to(device)
    basis = basis_on(T.params, device)
    A, _, E = N.cell_tables(nc, NSTEPS, th, basis)
    ties = torch.zeros(1, dtype=torch.int64, device=device)
    out = N.integrate(nc, NSTEPS, P, E, ties=ties)
    fp64_lookups = int(ties.item())
    cot = torch.randn(out.shape, generator=torch.Generator().manual_seed(1)).to(device)
    ws = torch.empty(N.load().cpab_backward_workspace(2, N._ints(nc), NSTEPS, P.shape[1], 512),
                     dtype=torch.uint8, device=device)
    fwd = lambda: N.integrate(nc, NSTEPS, P, E)
    bwd = lambda: N.backward(nc, NSTEPS, 0, P, A, E, basis, cot, workspace=ws)
    for _ in range(2):
        fwd()
        bwd()
    n = max(2, steps // 3)
    tf, tb = time_events(fwd, n, flush), time_events(bwd, n, flush)
    pts_n = 512 * 512 * 512
    # sample: 8 theta of each group x 1,024 grid points
    rows = torch.cat([torch.arange(0, 8), torch.arange(256, 264)])
    cols = torch.tensor(np.sort(np.random.default_rng(2).choice(512 * 512, 1024, replace=False)))
    Ps = P[:, cols.to(device)].contiguous()
    errs = {}
    for name, r in (('large_velocities', rows[:8]), ('near_identity', rows[8:])):
        o, c = N.integrate_trace(nc, NSTEPS, Ps, E[r.to(device)].contiguous())
        errs[name] = trajectory_errors(T.params.basis, theta[r].numpy(), Ps.cpu().numpy(), nc,
                                       o.cpu().numpy(), c.cpu().numpy())
    del out, cot, ws
    torch.cuda.empty_cache()
    return {'workload': 'transform_grid, tess [8,8] free, 256 theta ~ N(0,9I) + 256 theta ~ '
                        '1e-6 N(0,I), 512^2 grid per theta (134 M trajectories); backward: '
                        'dtheta (reference gradient, d = 234) for a N(0,1) cotangent',
            'forward_ms': sum(tf) / len(tf),
            'forward_points_per_s': pts_n / (sum(tf) / len(tf) / 1e3),
            'backward_ms': sum(tb) / len(tb),
            'fwd_bwd_points_per_s': pts_n / ((sum(tf) / len(tf) + sum(tb) / len(tb)) / 1e3),
            'fp64_path_lookups': fp64_lookups, 'lookups': pts_n * NSTEPS,
            'error_vs_fp64': errs}


CPU_SAMPLE_IMAGES, CPU_STEPS = 4, 3


def cpu_sample(n_img, given=None):
    """The headline inputs of the first n_img images on the host, plus the
    tables the reference's CPU op takes.  `given` = (theta, data, target) of
    the GPU run; otherwise they are rebuilt with the same seeds, the target
    being the images warped by the second theta (reference step maps and
    interpolation through the oracle; not timed)."""
    from oracle.oracle import Oracle, step_maps_fp64
    from libcpab_gb300.tessellation import make_tessellation
    basis = make_tessellation(NC, True, False).B
    d = basis.shape[1]
    lin = np.linspace(0, 1, SIZE, dtype=np.float32)
    gx, gy = np.meshgrid(lin, lin, indexing='xy')
    grid = np.ascontiguousarray(np.stack([gx.reshape(-1), gy.reshape(-1)]), dtype=np.float32)

    def tables(th):
        Tm = step_maps_fp64(basis, th, 2, NSTEPS)[:, :, :2, :].astype(np.float32)
        As = (basis @ th.astype(np.float64).T).T.reshape(th.shape[0], -1, 2, 3).astype(np.float32)
        return Tm, As
    if given is not None:
        th, data, target = (np.ascontiguousarray(x[:n_img].numpy()) for x in given)
    else:
        th = (THETA_STD * torch.randn(BATCH, d, generator=torch.Generator().manual_seed(0)))
        th = th[:n_img].numpy()
        raw = torch.rand(BATCH, CHANNELS, SIZE, SIZE, generator=torch.Generator().manual_seed(1))
        data = F.avg_pool2d(raw, kernel_size=5, stride=1, padding=2, count_include_pad=False)
        data = np.ascontiguousarray(data[:n_img].numpy())
        th2 = THETA_STD * torch.randn(BATCH, d, generator=torch.Generator().manual_seed(2))
        T2, _ = tables(th2[:n_img].numpy())
        orc = Oracle()
        target = orc.interpolate(data, orc.forward(NC, NSTEPS, grid, T2), [SIZE, SIZE])
    Tm, As = tables(th)
    Bs = basis.T.reshape(d, -1, 2, 3).astype(np.float32)
    return {'theta': th, 'data': data, 'target': np.ascontiguousarray(target, dtype=np.float32),
            'grid': grid, 'T': Tm, 'A': As, 'B': Bs, 'basis': basis,
            'n_total': BATCH * CHANNELS * SIZE * SIZE}


def cpu_reference_step(s, orc, ref, threads):
    """One step of the reference's CPU path on the sample: the integration
    forward, the interpolation, its backward, the analytic-gradient backward
    and its contraction.  The integration ops are the reference's own
    libcpab/core/cpab_ops.cpp (oracle/_ref, run on `threads` host threads
    over (theta, point-chunk) slices) when it is built, else their C
    restatement; the interpolation is the C restatement of
    libcpab/pytorch/interpolation.py (OpenMP)."""
    if ref is not None:
        out_grid = ref.forward_threaded(NC, NSTEPS, s['grid'], s['T'], threads)
    else:
        out_grid = orc.forward(NC, NSTEPS, s['grid'], s['T'])
    out = orc.interpolate(s['data'], out_grid, [SIZE, SIZE])
    gout = (2.0 * (out - s['target']) / s['n_total']).astype(np.float32)
    ddata, dgrid = orc.interpolate_backward(s['data'], out_grid, [SIZE, SIZE], gout)
    if ref is not None:
        dtheta = ref.dtheta_threaded(NC, NSTEPS, s['grid'], s['A'], s['B'], dgrid, threads)
    else:
        dtheta = orc.backward(NC, NSTEPS, s['grid'], s['A'], s['B'], dgrid)
    return dtheta, ddata


def run_cpu_baseline(steps, n_img, given=None):
    """Time the reference CPU path on n_img images (median of `steps`);
    returns (cpu_baseline dict, sample)."""
    from oracle.oracle import Oracle, RefLib
    orc = Oracle()
    threads = orc.num_threads()
    try:
        ref, kind = RefLib(), 'reference'
    except (OSError, FileNotFoundError):
        ref, kind = None, 'port'
    s = cpu_sample(n_img, given)
    times = []
    for _ in range(max(1, steps)):
        t0 = time.perf_counter()
        cpu_reference_step(s, orc, ref, threads)
        times.append(time.perf_counter() - t0)
    pts = n_img * SIZE * SIZE
    what = ("the reference's own libcpab/core/cpab_ops.cpp forward and analytic-gradient ops "
            "(oracle/_ref) on %d threads over (theta, point-chunk) slices" % threads
            if ref is not None else
            "the C restatement of libcpab/core/cpab_ops.cpp (oracle/, OpenMP, %d threads)"
            % threads)
    cb = {'value': pts / statistics.median(times), 'unit': 'points/s', 'cores': threads,
          'kind': kind, 'seconds_per_step': times,
          'sample': '%d of 64 images (%d points) per step, median of %d steps, loss = MSE '
                    'against the second-theta warp; %s; interpolation and its backward: the C '
                    'restatement of libcpab/pytorch/interpolation.py' % (n_img, pts,
                                                                         len(times), what)}
    return cb, s


def check_vs_fp64(s, chk):
    """The GPU's results on the sample images of the timed step, checked:
    trajectories against the FP64 oracle of the same scheme (C++ cell rules,
    boundary ties classified), the warped images against the reference's
    interpolation of the GPU's grid, dtheta and d(data) against the
    reference's gradient algorithm (C restatement) on the GPU's grid.
    chk: out [n, 2, nP] and cells [n, nP, 50] (traced integration), image
    [n, C, H, W], dtheta [n, d], ddata [n, C, H, W]."""
    from oracle.oracle import Oracle, numpy_transform_grid
    orc = Oracle()
    out, cells = chk['out'], chk['cells']
    ref, cells64, marg = numpy_transform_grid(s['basis'], s['theta'], s['grid'], NC, NSTEPS,
                                              return_cells=True, return_margin='steps',
                                              semantics='cpp')
    diff = cells != cells64
    tie = diff.any(axis=2)
    err = np.abs(out - ref).max(axis=1)
    first = diff.argmax(axis=2)
    ti, pi = np.nonzero(tie)
    fm = marg[ti, pi, first[ti, pi]] if ti.size else np.zeros(0)
    clean = err[~tie]
    img = orc.interpolate(s['data'], out, [SIZE, SIZE])
    gout = (2.0 * (img - s['target']) / s['n_total']).astype(np.float32)
    dd_ref, dgrid = orc.interpolate_backward(s['data'], out, [SIZE, SIZE], gout)
    dth_ref = orc.backward(NC, NSTEPS, s['grid'], s['A'], s['B'], dgrid)
    rel = lambda a, b: float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-30))
    r = {'sample': '%d of 64 images: %d trajectories of the timed inputs' % (out.shape[0],
                                                                            err.size),
         'clean_max_err': float(clean.max()) if clean.size else 0.0,
         'clean_p99_err': float(np.quantile(clean, 0.99)) if clean.size else 0.0,
         'tie_trajectories': int(tie.sum()),
         'tie_first_margin_max': float(fm.max()) if fm.size else 0.0,
         'image_max_abs_diff_vs_reference_interpolation': float(np.abs(chk['image'] - img).max()),
         'dtheta_rel_err_vs_reference_gradient': rel(chk['dtheta'], dth_ref),
         'ddata_rel_err_vs_reference': rel(chk['ddata'], dd_ref),
         'gates': 'point error <= 1e-5 on trajectories with the FP64 oracle\'s cells, every '
                  'other trajectory first diverging within 1e-6 of a decision boundary; '
                  'dtheta <= 1e-4 and d(data) <= 1e-5 relative to the reference algorithm '
                  'on the same warped grid'}
    r['pass'] = bool(r['clean_max_err'] <= 1e-5 and r['tie_first_margin_max'] < 1e-6 and
                     r['dtheta_rel_err_vs_reference_gradient'] <= 1e-4 and
                     r['ddata_rel_err_vs_reference'] <= 1e-5)
    return r


def run_cpu_numpy(n_img=1):
    """The reference's numpy backend (FP64, libcpab/numpy/transformer.py:22-61),
    restated in oracle/oracle.py, timed on its transform_grid of n_img images'
    224^2 grids.  Forward only: that backend has no gradient."""
    from oracle.oracle import numpy_transform_grid
    from libcpab_gb300.tessellation import make_tessellation
    B = make_tessellation(NC, True, False).B
    theta = THETA_STD * torch.randn(BATCH, B.shape[1], generator=torch.Generator().manual_seed(0))
    lin = np.linspace(0, 1, SIZE)
    gx, gy = np.meshgrid(lin, lin, indexing='xy')
    grid = np.stack([gx.reshape(-1), gy.reshape(-1)])
    t0 = time.perf_counter()
    numpy_transform_grid(B, theta[:n_img].numpy(), grid, NC, NSTEPS)
    dt = time.perf_counter() - t0
    pts = n_img * SIZE * SIZE
    return {'value': pts / dt, 'unit': 'points/s', 'cores': 1, 'kind': 'port',
            'sample': '%d of 64 theta x 224^2 grid points, transform_grid forward only (the '
                      'numpy backend has no gradient), one run' % n_img}


def main():
    args = parse()
    rank, world, _ = dist_env()
    if args.impl == 'reference':
        if rank != 0:
            return
        # a bounded sample per step (the reference's CPU path is ~1e4x slower
        # than the GPU): median of a few steps after one warm-up step
        steps = max(CPU_STEPS, min(args.steps, 5))
        run_cpu_baseline(1, args.cpu_sample_images)
        cb, _ = run_cpu_baseline(steps, args.cpu_sample_images)
        v = cb['value']
        line = {'impl': 'reference', 'metric': METRIC, 'value': v, 'unit': 'points/s',
                'n_gpus': args.gpus, 'steps': args.steps, 'warmup': args.warmup,
                'higher_is_better': True, 'scaling': 'weak', 'vs_baseline': None,
                'dtype': 'f32', 'data': 'synthetic',
                'config': {**workload_config(BATCH), 'parallelism': 'cpu',
                           'step': "the reference's CPU implementation on a sample of the "
                                   "batch (%d steps timed, median), see cpu_baseline.sample"
                                   % steps},
                'cpu_baseline': cb,
                'e2e': {'value': v, 'unit': 'points/s', 'h2d_bytes_per_step': 0,
                        'd2h_bytes_per_step': 0}}
        print(json.dumps(line))
        return
    if args.leg != 'all':
        device = torch.device('cuda', 0)
        torch.cuda.set_device(device)
        flush_buf = torch.empty(2 * L2_BYTES // 4, dtype=torch.float32, device=device)
        flush = lambda: flush_buf.fill_(1.0)
        fn = {'ragged': lambda: run_ragged(device, args.steps, flush, tune=not args.no_tune),
              'volume': lambda: run_volume(device, args.steps, flush, tune=not args.no_tune),
              'interp': lambda: run_interp_sweep(device, args.steps, flush),
              'aligner': lambda: run_aligner(device),
              'exact': lambda: run_exact_flow(device, args.steps, flush),
              'cfg1': lambda: run_cfg1(device, args.steps, flush),
              'cfg5': lambda: run_cfg5(device, args.steps, flush),
              'points': lambda: run_ragged_points(device, args.steps, flush,
                                                  tune=not args.no_tune),
              'mixed': lambda: run_mixed_images(device, args.steps, flush),
              'plain': lambda: run_plain_leg(device, args.steps, flush)}[args.leg]
        print(json.dumps({'leg': args.leg, 'result': fn()}))
        return
    res = run_gb300(args)
    if rank == 0 and res is not None:
        check = res.pop('_check', None)
        if world == 1 and not args.no_cpu_baseline:
            cb, sample = run_cpu_baseline(CPU_STEPS, args.cpu_sample_images,
                                          given=check['inputs'])
            res['cpu_baseline'] = cb
            res['error_vs_fp64'] = check_vs_fp64(sample, check)
            res['cpu_numpy_forward'] = run_cpu_numpy()
        print(json.dumps(res))


if __name__ == '__main__':
    main()
