#!/usr/bin/env python
"""Benchmark of the HCIPy diffraction hot path on GB300: the Lyot-coronagraph precision workload.

Workload (one "propagation" = one step): a 2048^2 circular pupil with seeded
Zernike 2-100 aberrations at 1 nm RMS, MFT to a 512^2 focal-plane-mask grid
(q=8, num_airy=32), occulter of radius 4 lambda/D, Babinet subtraction, Lyot
stop 0.9 D, final MFT to a 512^2 focal grid: three 2048^2 <-> 512^2 matrix
Fourier transforms (8,053,063,680 complex MACs = 64.42 GFLOP per propagation).

Prints one JSON line (rank 0).  ``--impl ours`` (default) times the CUDA path:
``value`` with inputs resident in HBM and L2 flushed between steps (a 256 MiB
write outside the per-step CUDA events); ``e2e`` through the public API with
the pupil field copied from pinned host memory and the final image copied
back inside the timed region.  ``--impl reference`` times the reference
algorithm's CPU port (oracle.optics.LyotChain, matrices precomputed as in the
reference's default configuration) on all host cores.
"""
import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = 'MFT propagations/s & adjoint grad steps/s at ≤1e-11 contrast err vs FP64'
UNIT = 'propagations/s'
L2_FLUSH_BYTES = 256 << 20
NI_BOUND = 1e-11  # the metric's contrast-error condition: max |NI - NI_fp64| over the dark hole


def parse_args():
    p = argparse.ArgumentParser()
    p.add_argument('--gpus', type=int, default=1)
    p.add_argument('--steps', type=int, default=200)
    p.add_argument('--warmup', type=int, default=10)
    p.add_argument('--impl', choices=['ours', 'reference'], default='ours')
    p.add_argument('--precision', choices=['fp32', 'split'], default='split')
    p.add_argument('--pupil', type=int, default=2048)
    p.add_argument('--no-cpu-baseline', action='store_true')
    p.add_argument('--cpu-seconds', type=float, default=10.0)
    p.add_argument('--grad-steps', type=int, default=20, help='timed DM-gradient steps (0: skip that leg)')
    p.add_argument('--no-atmosphere', action='store_true', help='skip the atmospheric-layer leg')
    p.add_argument('--no-graph', action='store_true', help='launch the step from Python instead of a CUDA graph')
    p.add_argument('--no-autotune', action='store_true', help='built-in tile choice instead of measured tiles')
    p.add_argument('--no-small', action='store_true',
                   help='skip the probe, EFC, 256^2 Fraunhofer, FFT-family, pyramid and vortex legs')
    p.add_argument('--broadband-frames', type=int, default=256,
                   help='frames of the broadband-through-turbulence leg (0: skip it)')
    p.add_argument('--lyot-batch', type=int, default=8,
                   help='fields per step of the batched Lyot leg, FP32 and split (0: skip it)')
    return p.parse_args()


def workload(args):
    from hcipy_gb300 import workloads
    return workloads.lyot_workload(pupil_n=args.pupil)


def flops_per_propagation(w):
    from hcipy_gb300.workloads import mft_complex_macs as mft_cmacs
    nx, ny = (int(d) for d in w['pupil'].dims)
    nu, nv = (int(d) for d in w['fpm_grid'].dims)
    fu, fv = (int(d) for d in w['focal'].dims)
    cmacs = 2 * mft_cmacs(nx, ny, nu, nv) + mft_cmacs(nx, ny, fu, fv)
    return cmacs, 8 * cmacs


def oracle_grid(g):
    from oracle.grids import RegularGrid
    return RegularGrid(g.delta, g.dims, g.zero)


# ---------------------------------------------------------------------------
# Clock sampling (nvidia-smi during the timed region)
# ---------------------------------------------------------------------------

class ClockSampler(object):
    FIELDS = ('clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,'
              'clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,'
              'clocks_event_reasons.sw_power_cap')

    def __init__(self, bus_id=None):
        self.bus_id = bus_id
        self.proc = None
        self.lines = []

    def start(self):
        cmd = ['nvidia-smi', '--query-gpu=' + self.FIELDS, '--format=csv,noheader,nounits', '-lms', '100']
        if self.bus_id:
            cmd[1:1] = ['-i', self.bus_id]
        try:
            self.proc = subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (OSError, ValueError):
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

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
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(',')]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                smax.append(float(parts[1]))
            except ValueError:
                continue
            for name, val in zip(('hw_slowdown', 'hw_thermal_slowdown', 'sw_thermal_slowdown', 'sw_power_cap'),
                                 parts[4:8]):
                if val.lower().startswith('active'):
                    reasons.add(name)
        if not sm:
            return {'sm_mhz': None, 'sm_max_mhz': None, 'reasons': [], 'samples': 0}
        return {'sm_mhz': statistics.median(sm), 'sm_max_mhz': max(smax), 'reasons': sorted(reasons),
                'samples': len(sm)}


def bus_id_of(dev):
    import torch
    try:
        p = torch.cuda.get_device_properties(dev)
        return '%08x:%02x:%02x.0' % (p.pci_domain_id, p.pci_bus_id, p.pci_device_id)
    except Exception:
        return None


# ---------------------------------------------------------------------------
# CPU side: the reference algorithm's port
# ---------------------------------------------------------------------------

def cpu_port_time(w, dtype, seconds, min_iters=1):
    """Propagations/s of oracle.optics.LyotChain on the host cores, over a bounded sample."""
    from oracle import optics
    chain = optics.LyotChain(oracle_grid(w['pupil']), oracle_grid(w['fpm_grid']), oracle_grid(w['focal']),
                             w['fpm'], w['stop'], dtype=dtype)
    e = w['E'].astype(dtype)
    chain(e)  # warm caches / BLAS threads
    n = 0
    t0 = time.perf_counter()
    while True:
        chain(e)
        n += 1
        if n >= min_iters and time.perf_counter() - t0 >= seconds:
            break
    dt = time.perf_counter() - t0
    return n / dt, n, dt


def host_cores():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


# ---------------------------------------------------------------------------
# Reference arm
# ---------------------------------------------------------------------------

def run_reference(args, rank, world):
    if rank != 0:
        return
    w = workload(args)
    from oracle import optics
    chain = optics.LyotChain(oracle_grid(w['pupil']), oracle_grid(w['fpm_grid']), oracle_grid(w['focal']),
                             w['fpm'], w['stop'], dtype=np.complex64)
    e = w['E'].astype(np.complex64)
    for _ in range(args.warmup):
        chain(e)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        chain(e)
    dt = time.perf_counter() - t0
    value = args.steps / dt
    cores = host_cores()
    line = {
        'impl': 'reference', 'metric': METRIC, 'value': value, 'unit': UNIT, 'n_gpus': args.gpus,
        'steps': args.steps, 'warmup': args.warmup, 'ms_per_step': 1e3 * dt / args.steps,
        'higher_is_better': True, 'scaling': 'weak', 'vs_baseline': None, 'dtype': 'fp32', 'data': 'synthetic',
        'config': {'workload': 'lyot-coronagraph 2048^2 pupil -> 512^2 FPM grid -> 512^2 image (3 MFTs)',
                   'pupil': args.pupil, 'fpm_grid': 512, 'image': 512, 'batch': 1, 'field_dtype': 'complex64'},
        'cpu_baseline': {'value': value, 'unit': UNIT, 'cores': cores, 'kind': 'port',
                         'sample': '%d propagations (the full workload) after %d warm-up, numpy/OpenBLAS cgemm '
                                   'with matrices precomputed' % (args.steps, args.warmup)},
        'e2e': {'value': value, 'unit': UNIT, 'h2d_bytes_per_step': 0, 'd2h_bytes_per_step': 0},
    }
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# Our arm
# ---------------------------------------------------------------------------

def dark_hole_error(img, ref_img, focal, aperture_peak):
    from hcipy_gb300 import workloads
    mask = workloads.dark_hole_mask(focal)
    ni = np.abs(img.astype(np.complex128))**2 / aperture_peak
    ni_ref = np.abs(ref_img)**2 / aperture_peak
    d = np.abs(ni - ni_ref)[mask]
    return float(d.max()), float(d.mean()), float(ni_ref[mask].mean())


def run_grad(args, dev):
    """Adjoint gradient steps: 64 DM command vectors -> Lyot coronagraph -> image intensity over a half annulus;
    one step = loss + gradient in all actuators through the device adjoints.  Returns the JSON object."""
    import torch
    import hcipy_gb300 as hg
    from hcipy_gb300 import workloads
    from oracle import optics
    w = workloads.dm_gradient_workload()
    pupil, fpm_grid, focal = w['pupil'], w['fpm_grid'], w['focal']
    lyot = hg.LyotCoronagraph(pupil, hg.Field(w['fpm'], fpm_grid), hg.Field(w['stop'], pupil),
                              precision=args.precision)
    prop = hg.FraunhoferPropagator(pupil, focal, precision=args.precision)
    dm = hg.DeformableMirror(w['influence'])
    e0 = torch.from_numpy(w['aperture'].astype(np.complex64)).to(dev)
    roi = torch.from_numpy(w['roi'].astype(np.float32)).to(dev)
    a0 = torch.from_numpy(w['actuators'].astype(np.float32)).to(dev)

    def step():
        a = a0.clone().requires_grad_(True)
        dm.actuators = a
        e = dm.forward(hg.Wavefront(hg.Field(e0, pupil), 1.0))
        img = prop.forward(lyot.forward(e)).electric_field.data
        loss = hg.intensity_sum(img, roi).sum()  # compensated dark-hole sums, fused, with their own backward
        loss.backward()
        return loss, a.grad

    hg.autotune(not args.no_autotune)
    for _ in range(3):
        step()
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream()
    t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    launches0 = hg.launch_count()
    t0.record(stream)
    for _ in range(args.grad_steps):
        loss, grad = step()
    t1.record(stream)
    t1.synchronize()
    ms = t0.elapsed_time(t1) / args.grad_steps
    launches = (hg.launch_count() - launches0) / args.grad_steps

    # accuracy: the float64 oracle gradient of the first command vectors
    from oracle.grids import RegularGrid
    og = lambda g: RegularGrid(g.delta, g.dims, g.zero)  # noqa: E731
    chain = optics.LyotChain(og(pupil), og(fpm_grid), og(focal), w['fpm'], w['stop'])
    m = w['influence'].transformation_matrix
    nv = 2
    g_dev = grad[:nv].double().cpu().numpy()
    errs = []
    for v in range(nv):
        _, g_ref = optics.dm_lyot_loss_grad(chain, m, w['aperture'], w['actuators'][v], w['roi'])
        errs.append(float(np.linalg.norm(g_dev[v] - g_ref) / np.linalg.norm(g_ref)))
    # CPU baseline: the same adjoint gradient with the oracle (complex64 numpy/OpenBLAS), per command vector
    chain64 = optics.LyotChain(og(pupil), og(fpm_grid), og(focal), w['fpm'], w['stop'], dtype=np.complex64)
    n, t_start = 0, time.perf_counter()
    while n < 1 or time.perf_counter() - t_start < args.cpu_seconds / 2:
        optics.dm_lyot_loss_grad(chain64, m, w['aperture'], w['actuators'][n % len(w['actuators'])], w['roi'])
        n += 1
    cpu_dt = time.perf_counter() - t_start
    nvec = w['actuators'].shape[0]
    return {
        'metric': 'adjoint grad steps/s', 'value': 1000.0 / ms, 'unit': 'grad steps/s', 'ms_per_step': ms,
        'steps': args.grad_steps, 'gpu_launches_per_step': launches,
        'config': {'workload': 'DM (34x34 Gaussian, %d illuminated actuators) -> Lyot coronagraph -> image '
                               'intensity over 3-12 lambda/D, x > 0; loss + gradient' % w['influence'].num_modes,
                   'pupil': int(pupil.dims[0]), 'fpm_grid': int(fpm_grid.dims[0]), 'image': int(focal.dims[0]),
                   'command_vectors': nvec, 'precision': args.precision,
                   'l2': 'not flushed; a step moves >1 GB (64 fields of 512^2, complex128 intermediates)'},
        'accuracy': {'grad_rel_l2_err_max': max(errs), 'vectors_checked': nv, 'against': 'float64 oracle adjoint'},
        'cpu_baseline': {'value': n / cpu_dt / nvec, 'unit': 'grad steps/s', 'cores': host_cores(), 'kind': 'port',
                         'sample': '%d command vectors in %.1f s (oracle adjoint gradient, complex64 numpy/OpenBLAS; '
                                   'the reference has no gradient)' % (n, cpu_dt)},
    }


def run_atmosphere(args, dev, peaks):
    """Infinite atmospheric layer at the broadband workload's size: 1024^2 screen over 8 m, float32 device
    matrices, wind 25 m/s, 1 ms frames (3.2 pixel steps per frame).  Times one extrusion (the A . stencil +
    B . noise update) and one quintic shift with CUDA events; the extrusion streams A and B from HBM."""
    import torch
    import hcipy_gb300 as hg
    from hcipy_gb300 import _lib
    pupil = hg.make_pupil_grid(1024, 8.0)
    t0 = time.perf_counter()
    layer = hg.InfiniteAtmosphericLayer(pupil, hg.Cn_squared_from_fried_parameter(0.1, 500e-9), L0=25,
                                        velocity=25.0, seed=5, dtype=torch.float32)
    init_s = time.perf_counter() - t0
    noise = torch.randn(64, layer.B_horizontal.shape[1], device=dev)
    for i in range(4):
        layer._extrude('right', noise[i])
    taps = np.array([0.0, 0.0, 0.0, 1.0, 0.0, 0.0, 0.0])
    torch.cuda.synchronize()
    # kernel times: CUDA events around each launch on its stream (the Python calls between launches are not
    # counted, so a launch-bound loop does not hide the kernel's own time)
    n = 60
    _lib.trace_read(_lib.HX_TRACE_ATMOSPHERE, reset=True)
    _lib.trace_enable(True)
    for i in range(n):
        layer._extrude('right', noise[i % 64])
    torch.cuda.synchronize()
    _lib.trace_enable(False)
    k, ms, _ = _lib.trace_read(_lib.HX_TRACE_ATMOSPHERE, reset=True)
    ext_us = ms / max(k, 1) * 1e3
    _lib.trace_enable(True)
    for i in range(n):
        layer._shift(taps, taps)
    torch.cuda.synchronize()
    _lib.trace_enable(False)
    k, ms, _ = _lib.trace_read(_lib.HX_TRACE_ATMOSPHERE, reset=True)
    shift_us = ms / max(k, 1) * 1e3
    ab_bytes = 4 * (layer.A_horizontal.size + layer.B_horizontal.size)
    hbm = peaks.get('hbm_gbs', 6800.0)
    frames = 20
    t_frame0 = torch.cuda.Event(enable_timing=True)
    t_frame1 = torch.cuda.Event(enable_timing=True)
    t_frame0.record()
    for f in range(frames):
        layer.evolve_until((f + 1) * 1e-3)
    t_frame1.record()
    t_frame1.synchronize()
    frame_ms = t_frame0.elapsed_time(t_frame1) / frames
    multi = time_multilayer(dev, hbm)
    from oracle import atmosphere as oatm
    screen = layer.achromatic_screen.data.double().cpu().numpy()
    rng = np.random.default_rng(0)
    cpu_n, c0 = 0, time.perf_counter()
    while cpu_n < 3 or time.perf_counter() - c0 < 2.0:
        screen = oatm.extrude(screen, (1024, 1024), 'right', layer.A_horizontal, layer.B_horizontal,
                              layer.stencil_left_idx, rng.standard_normal(layer.B_horizontal.shape[1]))
        cpu_n += 1
    cpu_ms = (time.perf_counter() - c0) / cpu_n * 1e3
    return {
        'layer': '1024^2 over 8 m, L0 25 m, v 25 m/s, float32 screen and A/B; init %.1f s on the host' % init_s,
        'extrusion_us': ext_us, 'extrusion_GBps': ab_bytes / (ext_us * 1e-6) / 1e9,
        'extrusion_frac_of_hbm': ab_bytes / (ext_us * 1e-6) / 1e9 / hbm,
        'extrusion_bytes': int(ab_bytes), 'shift_us': shift_us,
        'shift_GBps': 2 * 4 * pupil.size / (shift_us * 1e-6) / 1e9,
        'frame_ms': frame_ms, 'three_layers': multi,
        'frame': 'evolve_until for a 1 ms step: 3-4 extrusions (noise drawn on the host) and one shift, wall '
                 'time on the GPU including the host calls between launches',
        'kernel_timing': 'CUDA events around each extrusion / shift launch (hx_trace_enable)',
        'cpu_baseline_ms_per_extrusion': cpu_ms,
        'cpu_baseline': 'oracle extrusion (the reference algorithm: float64 GEMV + screen copy in numpy), %d steps '
                        'on the host' % cpu_n,
        'peak_note': 'hbm_gbs of measured' if 'hbm_gbs' in peaks else 'fallback',
    }


def time_multilayer(dev, hbm):
    """The broadband workload's three float32 1024^2 layers (r0 0.1/0.2/0.3 m, L0 25 m, winds 10/15/25 m/s):
    one extrusion of every layer in one launch (hx_atmosphere_extrude_layers) and the shift of the three screens
    with their sum in one pass (hx_atmosphere_shift_layers), CUDA events around each launch; then whole 1 ms
    frames of MultiLayerAtmosphere.evolve_until (host plans and noise draws included)."""
    import torch
    import hcipy_gb300 as hg
    from hcipy_gb300 import _lib, workloads
    w = workloads.broadband_turbulence_workload()
    pupil = w['pupil']
    layers = [hg.InfiniteAtmosphericLayer(pupil, hg.Cn_squared_from_fried_parameter(lay['r0'], 500e-9), L0=w['L0'],
                                          velocity=lay['velocity'], seed=lay['seed'], dtype=torch.float32)
              for lay in w['layers']]
    atm = hg.MultiLayerAtmosphere(layers)
    noise = torch.randn(3, layers[0].B_horizontal.shape[1], device=dev)
    lib, stream = _lib.lib(), _lib.stream_handle()

    def extrude_all():
        steps = (_lib.Extrusion * 3)(*[layer._extrusion('right', noise[i]) for i, layer in enumerate(layers)])
        _lib.check(lib.hx_atmosphere_extrude_layers(steps, 3, _lib.HX_F32, stream), 'hx_atmosphere_extrude_layers')
        for layer in layers:
            layer._moved('right')

    for _ in range(4):
        extrude_all()
    torch.cuda.synchronize()
    n = 60
    _lib.trace_read(_lib.HX_TRACE_ATMOSPHERE, reset=True)
    _lib.trace_enable(True)
    for _ in range(n):
        extrude_all()
    torch.cuda.synchronize()
    _lib.trace_enable(False)
    k, ms, _ = _lib.trace_read(_lib.HX_TRACE_ATMOSPHERE, reset=True)
    ext_us = ms / max(k, 1) * 1e3
    ab_bytes = 4.0 * sum(layer.A_horizontal.size + layer.B_horizontal.size for layer in layers)
    t = 0.0
    for _ in range(3):
        t += w['frame_time']
        atm.evolve_until(t)
    torch.cuda.synchronize()
    # the shift-and-sum pass alone: frames whose layers do not move (t unchanged) run only that launch
    _lib.trace_enable(True)
    for _ in range(n):
        atm.evolve_until(t)
    torch.cuda.synchronize()
    _lib.trace_enable(False)
    k, ms, _ = _lib.trace_read(_lib.HX_TRACE_ATMOSPHERE, reset=True)
    shift_us = ms / max(k, 1) * 1e3
    frames = 50
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    launches0 = hg.launch_count()
    ev0.record()
    for _ in range(frames):
        t += w['frame_time']
        atm.evolve_until(t)
    ev1.record()
    ev1.synchronize()
    return {
        'extrusion_us': ext_us, 'extrusion_bytes': int(ab_bytes),
        'extrusion_GBps': ab_bytes / (ext_us * 1e-6) / 1e9,
        'extrusion_frac_of_hbm': ab_bytes / (ext_us * 1e-6) / 1e9 / hbm,
        'extrusion': 'one step of each of the three layers in one launch (A 1024x3072 and B 1024x1024 float32 '
                     'each)',
        'shift_and_sum_us': shift_us,
        'shift_and_sum_GBps': 4.0 * 7 * pupil.size / (shift_us * 1e-6) / 1e9,
        'frame_ms': ev0.elapsed_time(ev1) / frames,
        'launches_per_frame': (hg.launch_count() - launches0) / frames,
    }


def run_broadband(args, dev, peaks):
    """Broadband imaging through turbulence: 21 wavelengths over 20 % bandwidth, each on its own diffraction-scaled
    focal grid (284^2 ... 232^2, q=4, 32 lambda0/lambda), a 1024^2 pupil of 8 m behind three float32 infinite
    layers (r0 0.1/0.2/0.3 m, L0 25 m, winds 10/15/25 m/s along x, seeds 5/6/7), 1 ms frames.  A frame evolves the
    layers (extrusions with host-drawn noise, quintic shifts, the summed screen) and replays one CUDA graph that
    holds, per wavelength, the phase of the summed screen and the matrix Fourier transform onto that wavelength's
    grid (in the split form the phase is applied while the transform slices its input); the split GEMMs run with
    the tiles the autotuner picked during the capture's warm-up."""
    import torch
    import hcipy_gb300 as hg
    from hcipy_gb300 import _lib, workloads
    w = workloads.broadband_turbulence_workload()
    pupil, wls, grids = w['pupil'], w['wavelengths'], w['focal_grids']
    t0 = time.perf_counter()
    layers = [hg.InfiniteAtmosphericLayer(pupil, hg.Cn_squared_from_fried_parameter(lay['r0'], 500e-9), L0=w['L0'],
                                          velocity=lay['velocity'], seed=lay['seed'], dtype=torch.float32)
              for lay in w['layers']]
    atm = hg.MultiLayerAtmosphere(layers)
    init_s = time.perf_counter() - t0
    ap = torch.from_numpy(w['aperture'].astype(np.complex64)).to(dev)
    nx, ny = (int(d) for d in pupil.dims)
    cmacs = sum(workloads.mft_complex_macs(nx, ny, int(g.dims[0]), int(g.dims[1])) for g in grids)
    frames, dt = args.broadband_frames, w['frame_time']
    legs = {}
    for precision in ('fp32', 'split'):
        imager = hg.BroadbandImager(pupil, wls, grids, focal_length=w['focal_length'], precision=precision,
                                    pre=atm.forward)
        atm.reset()
        imager.capture(ap)
        t = 0.0
        for _ in range(3):
            t += dt
            atm.evolve_until(t)
            imager.replay(ap)
        torch.cuda.synchronize()
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(6)]
        launches0 = hg.launch_count()
        ev[0].record()
        for _ in range(frames):
            t += dt
            atm.evolve_until(t)
            imager.replay(ap)
        ev[1].record()
        ev[1].synchronize()
        launches = hg.launch_count() - launches0
        # the two halves of a frame on their own
        ev[2].record()
        for _ in range(frames):
            imager.replay(ap)
        ev[3].record()
        for _ in range(frames):
            t += dt
            atm.evolve_until(t)
        ev[5].record()
        ev[5].synchronize()
        frame_ms = ev[0].elapsed_time(ev[1]) / frames
        graph_ms = ev[2].elapsed_time(ev[3]) / frames
        atm_ms = ev[3].elapsed_time(ev[5]) / frames
        # accuracy at the centre wavelength against the float64 oracle, on the field the device propagated
        k = len(wls) // 2
        from hcipy_gb300.kernels import apply_phase
        e_dev = apply_phase(ap, atm.combined_screen(), 1.0 / wls[k])
        img = imager.replay(ap)[k].cpu().numpy()
        from oracle import optics
        ref = optics.fraunhofer_forward(e_dev.cpu().numpy().astype(np.complex128), oracle_grid(pupil),
                                        oracle_grid(grids[k]), wavelength=wls[k], focal_length=w['focal_length'])
        peak_k = np.abs(optics.fraunhofer_forward(w['aperture'].astype(np.complex128), oracle_grid(pupil),
                                                  oracle_grid(grids[k]), wavelength=wls[k],
                                                  focal_length=w['focal_length'])).max()**2
        ni_err_k = np.abs(np.abs(img.astype(np.complex128))**2 - np.abs(ref)**2) / peak_k
        if precision == 'split':
            # the same graph with the wavelengths one after the other on one stream, for comparison
            seq = hg.BroadbandImager(pupil, wls, grids, focal_length=w['focal_length'], precision=precision,
                                     pre=atm.forward, streams=1).capture(ap)
            ev[2].record()
            for _ in range(frames):
                seq.replay(ap)
            ev[3].record()
            ev[3].synchronize()
            seq_ms = ev[2].elapsed_time(ev[3]) / frames
            del seq
        legs[precision] = {
            'frames_per_s': 1e3 / frame_ms, 'propagations_per_s': len(wls) * 1e3 / frame_ms, 'frame_ms': frame_ms,
            'graph_ms_per_frame': graph_ms, 'atmosphere_ms_per_frame': atm_ms,
            'tflops_in_graph': 8 * cmacs / (graph_ms * 1e-3) / 1e12,
            'launches_per_frame_outside_graph': launches / frames,
            'kernels_in_graph': int(imager.graph_kernels),
            'streams': imager.num_streams,
            'rel_err_vs_fp64': float(np.linalg.norm(img - ref) / np.linalg.norm(ref)),
            'ni_err_max_centre': float(ni_err_k.max()), 'ni_err_mean_centre': float(ni_err_k.mean()),
        }
        del imager
    # host baseline: the reference algorithm on the host cores (matrices precomputed per wavelength, as the
    # reference's propagator cache holds them), one frame's propagations over a bounded sample of wavelengths
    from oracle import fourier
    scr = atm.combined_screen().double().cpu().numpy()
    apn = w['aperture']
    x, y = pupil.separated_coords
    n_done, spent, c_all = 0, 0.0, time.perf_counter()
    for j in range(len(wls)):
        uv = oracle_grid(grids[j]).scaled(2 * np.pi / (w['focal_length'] * wls[j]))
        m1, m2 = fourier.mft_matrices(x, y, *uv.separated_coords)
        c1 = time.perf_counter()
        e = (apn * np.exp(1j * scr / wls[j])).reshape(ny, nx)
        m1 @ (e @ m2)
        spent += time.perf_counter() - c1
        n_done += 1
        if n_done >= 2 and time.perf_counter() - c_all > args.cpu_seconds / 2:
            break
    cpu_s_per_prop = spent / n_done
    return {
        'workload': '21 wavelengths over 20%% bandwidth, focal grids %d^2..%d^2 (q=4, 32 lambda0/lambda), 1024^2 '
                    'pupil of 8 m, 3 float32 infinite layers (r0 0.1/0.2/0.3 m, L0 25 m, 10/15/25 m/s along x, seeds '
                    '5/6/7), 1 ms '
                    'frames, %d frames' % (int(grids[0].dims[0]), int(grids[-1].dims[0]), frames),
        'fp32': legs['fp32'], 'split': legs['split'],
        'split_over_fp32': legs['split']['frames_per_s'] / legs['fp32']['frames_per_s'],
        'split_graph_ms_one_stream': seq_ms,
        'complex_macs_per_frame': int(cmacs),
        'layer_init_s': init_s,
        'timing': 'CUDA events on the stream around %d frames; graph_ms: the replays alone; atmosphere_ms: the '
                  'evolutions alone (host rng draws and launches included)' % frames,
        'cpu_baseline': {'propagations_per_s': 1.0 / cpu_s_per_prop, 'frames_per_s': 1.0 / (cpu_s_per_prop * len(wls)),
                         'cores': host_cores(), 'kind': 'port',
                         'sample': '%d of the 21 wavelengths: phase + two complex128 numpy GEMMs with precomputed '
                                   'matrices (matrix construction not timed)' % n_done},
    }


def run_lyot_batched(args, dev, ref_img, peak_img):
    """The Lyot workload with a batch of pupil fields per step (field 0 is the headline's field, the others carry
    extra seeded phase noise of 1 mrad RMS), FP32 and split precision, each step replayed from a CUDA graph: the
    batched form of the chain, where the transforms stack the fields into larger GEMMs.  The same graphs with one
    field per step give the single-field rates of both forms, measured side by side."""
    import torch
    import hcipy_gb300 as hg
    w = workload(args)
    pupil, fpm_grid, focal = w['pupil'], w['fpm_grid'], w['focal']
    nb = args.lyot_batch
    rng = np.random.default_rng(17)
    e = np.repeat(w['E'][None, :].astype(np.complex64), nb, axis=0)
    e[1:] *= np.exp(1j * 1e-3 * rng.standard_normal((nb - 1, pupil.size))).astype(np.complex64)
    e_dev = torch.from_numpy(e).to(dev)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)
    out = {'workload': 'lyot-coronagraph 2048^2 -> 512^2 FPM grid -> 512^2 image, %d fields per step' % nb,
           'batch': nb}
    for precision in ('fp32', 'split'):
        lyot = hg.LyotCoronagraph(pupil, hg.Field(w['fpm'], fpm_grid), hg.Field(w['stop'], pupil),
                                  precision=precision)
        prop = hg.FraunhoferPropagator(pupil, focal, precision=precision)

        def step(x):
            return prop.forward(lyot.forward(hg.Wavefront(hg.Field(x, pupil), 1.0))).electric_field.data

        hg.autotune(not args.no_autotune)

        def timed(x, steps):
            graph = hg.CapturedCall(step, x, warmup=3)
            res = graph(x)
            torch.cuda.synchronize()
            ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
            for i in range(steps):
                flush.fill_(float(i))
                ev[i][0].record()
                graph(x)
                ev[i][1].record()
            torch.cuda.synchronize()
            return res.clone(), sum(a.elapsed_time(b) for a, b in ev) / steps, int(graph.graph_kernels)

        img, ms, kernels = timed(e_dev, 10)
        _, ms1, _ = timed(e_dev[0].clone(), 20)
        leg = {'propagations_per_s': nb * 1e3 / ms, 'ms_per_step': ms, 'kernels_in_graph': kernels,
               'propagations_per_s_one_field': 1e3 / ms1}
        if ref_img is not None:
            leg['ni_err_max_field0'] = dark_hole_error(img[0].cpu().numpy(), ref_img, focal, peak_img)[0]
        out[precision] = leg
        del lyot, prop
    out['split_over_fp32'] = out['split']['propagations_per_s'] / out['fp32']['propagations_per_s']
    out['split_over_fp32_one_field'] = (out['split']['propagations_per_s_one_field'] /
                                        out['fp32']['propagations_per_s_one_field'])
    out['timing'] = 'CUDA events around each graph replay, L2 flushed between steps outside the events'
    return out


def time_efc_step(em, field, dz_dev, actuators, dev, steps=50):
    """hx_efc_step alone (dark-zone gather, float64 EFC-matrix product in float-float, update), CUDA events on
    the launching stream around each launch, L2 flushed between launches outside the events.  Algorithmic
    bytes: the matrix once, the gathered field values, indices, commands in and out."""
    import torch
    from hcipy_gb300 import _lib
    idx = torch.nonzero(dz_dev.reshape(-1)).reshape(-1).to(torch.int32).contiguous()
    m = em.to(torch.float64).contiguous()
    e = field.reshape(-1).contiguous()
    a = actuators.to(torch.float64).contiguous()
    out = torch.empty_like(a)
    nact, n_dz = int(m.shape[0]), int(idx.numel())
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream()
    lib = _lib.lib()

    def launch():
        _lib.check(lib.hx_efc_step(_lib.dptr(m), nact, n_dz, _lib.dptr(e), _lib.dtype_code(e.dtype), _lib.dptr(idx),
                                   _lib.dptr(a), 0.5, _lib.dptr(out), _lib.stream_handle()), 'hx_efc_step')

    for _ in range(3):
        launch()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    torch.cuda.synchronize()
    for i in range(steps):
        flush.fill_(float(i))
        ev[i][0].record(stream)
        launch()
        ev[i][1].record(stream)
    torch.cuda.synchronize()
    us = 1e3 * sum(x.elapsed_time(y) for x, y in ev) / steps
    nbytes = 8.0 * nact * 2 * n_dz + e.element_size() * n_dz + 4.0 * n_dz + 16.0 * nact
    peaks = {}
    try:
        with open(os.path.join(ROOT, 'MEASURED_PEAKS.json')) as f:
            peaks = json.load(f)
    except (OSError, ValueError):
        pass
    hbm = peaks.get('hbm_gbs', 6800.0)
    return {'matrix': [nact, 2 * n_dz], 'field_dtype': str(e.dtype).replace('torch.', ''), 'us_per_step': us,
            'algorithmic_bytes': nbytes, 'achieved_gbs': nbytes / (us * 1e-6) / 1e9,
            'frac_of_hbm': nbytes / (us * 1e-6) / 1e9 / hbm,
            'peak_note': 'hbm_gbs of measured' if 'hbm_gbs' in peaks else 'fallback',
            'timing': 'CUDA events around each launch, L2 flushed between launches outside the events'}


def run_efc(args, dev):
    """Electric-field conjugation on the gradient workload's optics (512^2 pupil, 952-actuator DM, Lyot
    coronagraph, 256^2 image, dark zone = the 3-12 lambda/D half annulus): the poke Jacobian of every actuator
    (+-1e-3 lambda pokes: 1904 propagations, 64 actuators per call), its Tikhonov inverse (rcond 1e-2, float64
    SVD on the device) and ten EFC iterations (gain 0.5) against a seeded 0.02 rad RMS pupil aberration."""
    import torch
    import hcipy_gb300 as hg
    from hcipy_gb300 import workloads
    from oracle import optics
    w = workloads.dm_gradient_workload()
    pupil, fpm_grid, focal = w['pupil'], w['fpm_grid'], w['focal']
    split = args.precision == 'split'
    lyot = hg.LyotCoronagraph(pupil, hg.Field(w['fpm'], fpm_grid), hg.Field(w['stop'], pupil),
                              precision=args.precision)
    prop = hg.FraunhoferPropagator(pupil, focal, precision=args.precision)
    dm = hg.DeformableMirror(w['influence'], dtype=torch.float64 if split else torch.float32)
    cdt = torch.complex128 if split else torch.complex64
    rdt = torch.float64 if split else torch.float32
    ap = torch.from_numpy(w['aperture'].astype(np.complex128)).to(dev, cdt)
    rng = np.random.default_rng(21)
    ab = torch.from_numpy(w['aperture'] * np.exp(0.02j * rng.standard_normal(pupil.size))).to(dev, cdt)
    nact = w['influence'].num_modes
    dz = w['roi']

    def measure(e0):
        def f(cmds):
            dm.actuators = cmds
            return prop.forward(lyot.forward(dm.forward(hg.Wavefront(hg.Field(e0, pupil), 1.0)))).electric_field.data
        return f

    hg.autotune(not args.no_autotune)
    hg.poke_jacobian(measure(ap), dz, nact, 1e-3, batch=64, dtype=rdt)  # warm-up: plans, workspaces, tiles
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    jac = hg.poke_jacobian(measure(ap), dz, nact, 1e-3, batch=64, dtype=rdt)
    torch.cuda.synchronize()
    t_jac = time.perf_counter() - t0
    t_inv = []
    for _ in range(2):  # the first call also creates the process's solver handles
        t0 = time.perf_counter()
        em = hg.inverse_tikhonov(jac, 1e-2)
        torch.cuda.synchronize()
        t_inv.append(time.perf_counter() - t0)
    peak = float(prop.forward(hg.Wavefront(hg.Field(ap, pupil), 1.0)).electric_field.data.abs().max())**2
    dz_dev = torch.from_numpy(dz).to(dev)
    one = measure(ab)
    iters = 10
    hg.run_efc(lambda a: one(a[None])[0], dz, em, np.zeros(nact), 1, 0.5)  # warm-up: single-field plans, tiles
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    hist, fields = hg.run_efc(lambda a: one(a[None])[0], dz, em, np.zeros(nact), iters, 0.5)
    torch.cuda.synchronize()
    t_loop = time.perf_counter() - t0
    ni = [float((f[dz_dev].abs()**2).mean()) / peak for f in fields]
    step_leg = time_efc_step(em, fields[-1], dz_dev, hist[-1], dev)
    # host: the same pokes through the reference algorithm's port (complex128, matrices precomputed), a bounded
    # sample of actuators, extrapolated to all of them
    chain = optics.LyotChain(oracle_grid(pupil), oracle_grid(fpm_grid), oracle_grid(focal), w['fpm'], w['stop'])
    inf = w['influence'].transformation_matrix
    e0 = w['aperture'].astype(np.complex128)
    c0, done = time.perf_counter(), 0
    for i in range(nact):
        for a in (-1e-3, 1e-3):
            chain(optics.dm_forward(e0, inf[:, i].toarray().ravel() * a, 1.0))
        done += 1
        if time.perf_counter() - c0 > args.cpu_seconds / 2:
            break
    cpu_per_act = (time.perf_counter() - c0) / done
    return {
        'workload': '952-actuator DM on 512^2 -> Lyot (512^2 FPM grid) -> 256^2 image; dark zone 3-12 lambda/D, '
                    'x > 0 (%d pixels)' % int(dz.sum()),
        'precision': args.precision, 'jacobian_shape': list(jac.shape),
        'jacobian_s': t_jac, 'propagations_per_s_in_jacobian': 2 * nact / t_jac,
        'tikhonov_inverse_s': t_inv[1], 'tikhonov_first_call_s': t_inv[0], 'efc_iterations': iters, 'efc_ms_per_iteration': 1e3 * t_loop / iters,
        'dark_zone_ni_first_last': [ni[0], ni[-1]],
        'efc_step_kernel': step_leg,
        'timing': 'host wall clock with a device synchronize on both sides',
        'cpu_baseline': {'jacobian_s_estimate': cpu_per_act * nact, 'cores': host_cores(), 'kind': 'port',
                         'sample': '%d of %d actuators (2 pokes each) through the numpy port, complex128, '
                                   'extrapolated' % (done, nact)},
    }


def run_dm_probes(args, dev):
    """Pair-wise DM probing, the electric-field-conjugation measurement step: the unprobed field and four probe
    shapes applied with both signs (9 command vectors) through the DM (952 Gaussian actuators on a 512^2 pupil),
    the Lyot coronagraph (512^2 focal-plane-mask grid) and the lens (256^2 image), intensities out; the whole
    batch replayed from one CUDA graph (hcipy_gb300.CapturedCall) with new commands each iteration."""
    import torch
    import hcipy_gb300 as hg
    from hcipy_gb300 import workloads
    w = workloads.dm_gradient_workload()
    pupil, fpm_grid, focal = w['pupil'], w['fpm_grid'], w['focal']
    lyot = hg.LyotCoronagraph(pupil, hg.Field(w['fpm'], fpm_grid), hg.Field(w['stop'], pupil),
                              precision=args.precision)
    prop = hg.FraunhoferPropagator(pupil, focal, precision=args.precision)
    dm = hg.DeformableMirror(w['influence'])
    e0 = torch.from_numpy(w['aperture'].astype(np.complex64)).to(dev)
    nact = w['influence'].num_modes
    rng = np.random.default_rng(9)
    probes = rng.standard_normal((4, nact)) * 2e-3
    base = w['actuators'][0]
    cmds = [base] + [base + sgn * p for p in probes for sgn in (1, -1)]
    cmd = torch.from_numpy(np.asarray(cmds, np.float32)).to(dev)

    def measure(c):
        dm.actuators = c
        e = dm.forward(hg.Wavefront(hg.Field(e0, pupil), 1.0))
        img = prop.forward(lyot.forward(e)).electric_field.data
        return img.real**2 + img.imag**2

    hg.autotune(not args.no_autotune)
    direct = measure(cmd).clone()
    graph = hg.CapturedCall(measure, cmd)
    replay = graph(cmd).clone()
    same = bool(torch.equal(direct, replay))
    n = 50
    new = [cmd + 1e-4 * torch.randn_like(cmd) for _ in range(4)]
    torch.cuda.synchronize()
    t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    t0.record()
    for i in range(n):
        graph(new[i % 4])
    t1.record()
    t1.synchronize()
    ms = t0.elapsed_time(t1) / n
    return {
        'workload': '9 command vectors (unprobed + 4 probes x 2 signs) -> 952-actuator DM on 512^2 -> Lyot (512^2 '
                    'FPM grid) -> 256^2 intensity',
        'probe_sets_per_s': 1e3 / ms, 'propagations_per_s': 9 * 1e3 / ms, 'ms_per_probe_set': ms,
        'kernels_in_graph': int(graph.graph_kernels), 'graph_equals_direct': same, 'precision': args.precision,
    }


def run_small_fraunhofer(args, dev, peaks):
    """A 256^2 pupil (Zernike 2-21 at 0.1 rad RMS) onto a 128^2 focal grid (q=4, num_airy=16): 12,582,912 complex
    MACs per propagation, a launch-latency-bound size.  Propagations/s through FraunhoferPropagator.forward with
    Python launches and replayed from a CUDA graph of 64 propagations, FP32 and split precision."""
    import torch
    import hcipy_gb300 as hg
    from hcipy_gb300 import workloads
    from oracle import optics
    w = workloads.fraunhofer_workload()
    pupil, focal = w['pupil'], w['focal']
    e = torch.from_numpy(w['E'].astype(np.complex64)).to(dev)
    ref = optics.fraunhofer_forward(w['E'].astype(np.complex64).astype(np.complex128), oracle_grid(pupil),
                                    oracle_grid(focal))
    nx, ny = (int(d) for d in pupil.dims)
    cmacs = workloads.mft_complex_macs(nx, ny, int(focal.dims[0]), int(focal.dims[1]))
    out = {'workload': '256^2 pupil, Zernike 2-21 at 0.1 rad RMS -> 128^2 focal grid (q=4, num_airy=16)',
           'complex_macs': int(cmacs)}
    for precision in ('fp32', 'split'):
        prop = hg.FraunhoferPropagator(pupil, focal, precision=precision)
        wf = hg.Wavefront(hg.Field(e, pupil), 1.0)
        for _ in range(5):
            img = prop.forward(wf).electric_field.data
        torch.cuda.synchronize()
        n = 200
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
        ev[0].record()
        for _ in range(n):
            prop.forward(wf)
        ev[1].record()
        ev[1].synchronize()
        py_us = ev[0].elapsed_time(ev[1]) / n * 1e3
        graph = torch.cuda.CUDAGraph()
        side = torch.cuda.Stream()
        side.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(side):
            prop.forward(wf)
        torch.cuda.current_stream().wait_stream(side)
        per_graph = 64
        with torch.cuda.graph(graph):
            for _ in range(per_graph):
                prop.forward(wf)
        graph.replay()
        torch.cuda.synchronize()
        reps = 10
        ev[2].record()
        for _ in range(reps):
            graph.replay()
        ev[3].record()
        ev[3].synchronize()
        g_us = ev[2].elapsed_time(ev[3]) / (reps * per_graph) * 1e3
        err = float(np.linalg.norm(img.cpu().numpy() - ref) / np.linalg.norm(ref))
        out[precision] = {'propagations_per_s_python': 1e6 / py_us, 'propagations_per_s_graph': 1e6 / g_us,
                          'us_per_propagation_graph': g_us, 'tflops_graph': 8 * cmacs / (g_us * 1e-6) / 1e12,
                          'rel_err_vs_fp64': err}
    from oracle import fourier
    x, y = pupil.separated_coords
    uv = oracle_grid(focal)
    m1, m2 = fourier.mft_matrices(x, y, *uv.separated_coords)
    e_h = w['E'].astype(np.complex64).reshape(ny, nx)
    m1, m2 = m1.astype(np.complex64), m2.astype(np.complex64)
    k, c0 = 0, time.perf_counter()
    while k < 20 or time.perf_counter() - c0 < 1.0:
        m1 @ (e_h @ m2)
        k += 1
    out['cpu_baseline'] = {'propagations_per_s': k / (time.perf_counter() - c0), 'cores': host_cores(), 'kind': 'port',
                           'sample': '%d propagations, complex64 numpy GEMMs with precomputed matrices' % k}
    return out


def run_modulated_pyramid(args, dev):
    """The modulated pyramid wavefront sensor: a 256^2 pupil (Zernike 2-21 at 0.5 rad RMS) through 12 modulation
    steps of radius 3 lambda/D onto a 256^2 sensor plane of twice the pupil's extent (512^2 focal grid, q = 2),
    complex64 on the FP32 transforms; the tip-tilt method (the reference's default: every step tilted, then two
    transforms) and the shifted-pyramid method (one transform, a phase per step, one transform).  Frames/s with
    Python launches, the steps against the float64 oracle, and the oracle port timed on the host for one frame."""
    import torch
    import hcipy_gb300 as hg
    from hcipy_gb300 import workloads
    from oracle import optics
    from oracle.grids import make_pupil_grid as o_pupil
    n, steps, mod = 256, 12, 3.0
    pupil, wfs_grid = hg.make_pupil_grid(n, 1.0), hg.make_pupil_grid(n, 2.0)
    ap = workloads.circular_aperture(pupil, 1.0)
    e_h = ap * np.exp(1j * workloads.zernike_phase(pupil, 1.0, 2, 21, 0.5, 3))
    e = torch.from_numpy(e_h.astype(np.complex64)).to(dev)
    pwfs = hg.PyramidWavefrontSensorOptics(pupil, wfs_grid)
    po = optics.PyramidOptics(o_pupil(n, 1.0), o_pupil(n, 2.0), 1.0, 1.0, 1, lambda x: 1.5)
    nf = int(pwfs.focal_grid.dims[0])
    cmacs = steps * (workloads.mft_complex_macs(n, n, nf, nf) + workloads.mft_complex_macs(nf, nf, n, n))
    out = {'workload': '256^2 pupil, Zernike 2-21 at 0.5 rad RMS -> 12 modulation steps of 3 lambda/D -> 512^2 '
                       'focal grid -> 256^2 sensor plane, complex64', 'complex_macs_per_frame_tip_tilt': int(cmacs)}
    for name, fast in (('tip_tilt', False), ('shifted_pyramid', True)):
        m = hg.ModulatedPyramidWavefrontSensorOptics(pwfs, mod, num_steps=steps, fast_modulation_method=fast)
        wf = hg.Wavefront(hg.Field(e, pupil), 1.0)
        for _ in range(3):
            res = m.forward(wf)
        torch.cuda.synchronize()
        k = 30
        t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t0.record()
        for _ in range(k):
            m.forward(wf)
        t1.record()
        t1.synchronize()
        ms = t0.elapsed_time(t1) / k
        got = np.stack([w.electric_field.numpy() for w in res]).astype(np.complex128)
        ref = optics.modulated_pyramid_forward(po, e_h.astype(np.complex64).astype(np.complex128), 1.0, mod, steps,
                                               fast=fast)
        out[name] = {'frames_per_s': 1e3 / ms, 'ms_per_frame': ms, 'steps_per_s': steps * 1e3 / ms,
                     'rel_err_vs_fp64': float(np.linalg.norm(got - ref) / np.linalg.norm(ref))}
        if not fast:
            c0 = time.perf_counter()
            optics.modulated_pyramid_forward(po, e_h, 1.0, mod, steps)
            cpu_s = time.perf_counter() - c0
            out['cpu_baseline'] = {'frames_per_s': 1 / cpu_s, 'cores': host_cores(), 'kind': 'port',
                                   'sample': 'one frame of the tip-tilt method through the numpy port, complex128'}
    return out


def run_vortex(args, dev):
    """Multi-scale vortex coronagraphs on a 256^2 pupil with the reference's default sampling (charge 2, q = 1024,
    scaling factor 4, window 32: six levels, a 512^2 Fourier filter and five 256^2 <-> 128^2 MFT pairs), no Lyot
    stop: Lyot-plane fields/s with Python launches for the scalar vortex in complex64 and complex128 and for the
    vector vortex (its three scalar coronagraphs) in complex64, the plan times, the errors against the float64
    oracle and the oracle port timed on the host."""
    import torch
    import hcipy_gb300 as hg
    from hcipy_gb300 import workloads
    from oracle import optics
    from oracle.grids import make_pupil_grid as o_pupil
    n = 256
    pupil = hg.make_pupil_grid(n, 1.0)
    e_h = workloads.circular_aperture(pupil, 1.0) * np.exp(1j * workloads.zernike_phase(pupil, 1.0, 2, 21, 0.05, 5))
    out = {'workload': '256^2 pupil, Zernike 2-21 at 0.05 rad RMS, charge-2 vortex (q 1024, scaling factor 4, '
                       'window 32: 6 levels), Lyot plane without a stop'}

    def timed(fn, k=20):
        for _ in range(3):
            fn()
        torch.cuda.synchronize()
        t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t0.record()
        for _ in range(k):
            fn()
        t1.record()
        t1.synchronize()
        return t0.elapsed_time(t1) / k

    def rel(a, b):
        return float(np.linalg.norm(a - b) / np.linalg.norm(b))

    c0 = time.perf_counter()
    vc = hg.VortexCoronagraph(pupil, 2)
    torch.cuda.synchronize()
    out['scalar_plan_s'] = time.perf_counter() - c0
    oracle = optics.MultiScaleOptics(o_pupil(n, 1.0), optics.vortex_mask(2), 1024, 4, 32)
    for name, dtype in (('scalar_c64', np.complex64), ('scalar_c128', np.complex128)):
        wf = hg.Wavefront(hg.Field(torch.from_numpy(e_h.astype(dtype)).to(dev), pupil), 1.0)
        ms = timed(lambda: vc.forward(wf))
        got = vc.forward(wf).electric_field.numpy().astype(np.complex128)
        ref = oracle.propagate(e_h.astype(dtype).astype(np.complex128))
        out[name] = {'lyot_fields_per_s': 1e3 / ms, 'ms_per_field': ms, 'rel_err_vs_fp64': rel(got, ref)}
    vvc = hg.VectorVortexCoronagraph(2)
    wf = hg.Wavefront(hg.Field(torch.from_numpy(e_h.astype(np.complex64)).to(dev), pupil), 1.0)
    c0 = time.perf_counter()
    vvc.forward(wf)
    torch.cuda.synchronize()
    out['vector_plan_s'] = time.perf_counter() - c0
    ms = timed(lambda: vvc.forward(wf))
    got = vvc.forward(wf).electric_field.numpy().astype(np.complex128)
    ref = optics.MultiScaleOptics(o_pupil(n, 1.0), optics.vector_vortex_mask(2, np.pi), 1024, 4, 32).propagate(
        e_h.astype(np.complex64).astype(np.complex128))
    out['vector_c64'] = {'lyot_fields_per_s': 1e3 / ms, 'ms_per_field': ms, 'rel_err_vs_fp64': rel(got, ref)}
    k, c0 = 0, time.perf_counter()
    while k < 5 or time.perf_counter() - c0 < 1.0:
        oracle.propagate(e_h)
        k += 1
    out['cpu_baseline'] = {'lyot_fields_per_s': k / (time.perf_counter() - c0), 'cores': host_cores(), 'kind': 'port',
                           'sample': '%d scalar propagations through the numpy port, complex128' % k}
    return out


def run_fft_family(args, dev, peaks):
    """A 1024^2 pupil of 8 m behind a von Karman screen (r0 0.15 m, L0 20 m) at 1.6 um: the zero-padded FFT to
    4096^2 (q=4) and angular-spectrum propagation over 0.5 m and 5 m (2048^2 padded).  Per-call time with CUDA
    events, the line-FFT passes bracketed by events on their stream, and the HBM rate of the algorithmic bytes
    (input + output, complex64)."""
    import torch
    import hcipy_gb300 as hg
    from hcipy_gb300 import _lib, workloads
    w = workloads.turbulent_pupil_workload()
    pupil = w['pupil']
    e = torch.from_numpy(w['E'].astype(np.complex64)).to(dev)
    hbm = peaks.get('hbm_gbs', 6800.0)
    fft = hg.FastFourierTransform(pupil, q=4, fov=1)
    wf = hg.Wavefront(hg.Field(e, pupil), w['wavelength'])
    cases = [('fft_1024_to_4096', lambda: fft.forward(e), 8 * (pupil.size + fft.output_grid.size))]
    for d in (0.5, 5.0):
        asp = hg.AngularSpectrumPropagator(pupil, d)
        cases.append(('asp_%gm' % d, (lambda a: lambda: a.forward(wf))(asp), 8 * 2 * pupil.size))
    out = {'workload': '1024^2 pupil of 8 m, von Karman r0 0.15 m, L0 20 m, lambda 1.6 um; padded FFT q=4 -> 4096^2; '
                       'angular spectrum 0.5 m and 5 m (2048^2 padded)'}
    for name, fn, nbytes in cases:
        for _ in range(3):
            fn()
        torch.cuda.synchronize()
        n = 20
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        _lib.trace_read(_lib.HX_TRACE_FFT, reset=True)
        _lib.trace_enable(True)
        e0.record()
        for _ in range(n):
            fn()
        e1.record()
        e1.synchronize()
        _lib.trace_enable(False)
        k, ms, _ = _lib.trace_read(_lib.HX_TRACE_FFT, reset=True)
        call_us = e0.elapsed_time(e1) / n * 1e3
        pass_us = ms / n * 1e3
        out[name] = {'us_per_call': call_us, 'pass_us_per_call': pass_us, 'passes_per_call': k // n,
                     'algorithmic_bytes': int(nbytes), 'GBps': nbytes / (pass_us * 1e-6) / 1e9,
                     'frac_of_hbm': nbytes / (pass_us * 1e-6) / 1e9 / hbm}
    # accuracy of the padded FFT against the float64 oracle
    from oracle import fourier
    plan = fourier.FFTPlan(oracle_grid(pupil), 4, 1)
    ref = plan.forward(w['E'].astype(np.complex64).astype(np.complex128))
    got = fft.forward(e).numpy()
    out['fft_1024_to_4096']['rel_err_vs_fp64'] = float(np.linalg.norm(got - ref) / np.linalg.norm(ref))
    c0 = time.perf_counter()
    plan.forward(w['E'])
    out['cpu_baseline'] = {'fft_1024_to_4096_ms': (time.perf_counter() - c0) * 1e3, 'cores': 1, 'kind': 'port',
                           'sample': 'one padded FFT, numpy pocketfft on complex128 (the reference pads in complex128)'}
    out['peak_note'] = 'hbm_gbs of measured' if 'hbm_gbs' in peaks else 'fallback'
    return out


def max_over_ranks(value, dist, device):
    """The largest value over all ranks (a no-op without a process group): the whole job's time."""
    if dist is None:
        return float(value)
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def run_ours(args, rank, world, dist):
    import torch
    import hcipy_gb300 as hg

    dev = torch.device('cuda', int(os.environ.get('LOCAL_RANK', 0)))
    torch.cuda.set_device(dev)
    w = workload(args)
    pupil, fpm_grid, focal = w['pupil'], w['fpm_grid'], w['focal']
    cmacs, flops = flops_per_propagation(w)

    lyot = hg.LyotCoronagraph(pupil, hg.Field(w['fpm'], fpm_grid), hg.Field(w['stop'], pupil),
                              precision=args.precision)
    prop = hg.FraunhoferPropagator(pupil, focal, precision=args.precision)
    e_dev = torch.from_numpy(w['E'].astype(np.complex64)).to(dev)
    stream = torch.cuda.current_stream()

    def step(e):
        wf = hg.Wavefront(hg.Field(e, pupil), 1.0)
        return prop.forward(lyot.forward(wf)).electric_field.data

    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)
    # the warm-up measures the tile candidates of each GEMM shape once (not under a profiler, whose replays
    # distort the timings: --no-autotune keeps the built-in tile choice)
    hg.autotune(not args.no_autotune)
    for _ in range(max(args.warmup, 3)):
        img = step(e_dev)
    torch.cuda.synchronize()

    # -- the step as a CUDA graph: plans, workspaces and tiles exist after the warm-up -----------------
    graph = None
    if not args.no_graph:
        static_e = e_dev.clone()
        side = torch.cuda.Stream()
        side.wait_stream(stream)
        with torch.cuda.stream(side):
            for _ in range(2):
                step(static_e)
        stream.wait_stream(side)
        graph = torch.cuda.CUDAGraph()
        launches_captured = hg.launch_count()
        with torch.cuda.graph(graph):
            static_img = step(static_e)
        launches_per_replay = hg.launch_count() - launches_captured
        torch.cuda.synchronize()

    # -- device-resident timing: per-step events, L2 flushed between steps outside the events --------
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    sampler = ClockSampler(bus_id_of(dev))
    sampler.start()
    time.sleep(0.3)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    launches0 = hg.launch_count()
    wall0 = time.perf_counter()
    for i in range(args.steps):
        flush.fill_(float(i))
        starts[i].record(stream)
        if graph is not None:
            graph.replay()
        else:
            img = step(e_dev)
        ends[i].record(stream)
    torch.cuda.synchronize()
    wall = time.perf_counter() - wall0
    launches = hg.launch_count() - launches0 + (launches_per_replay * args.steps if graph is not None else 0)
    if graph is not None:
        img = static_img

    # -- kernel timing for the roofline: the same steps without the graph, CUDA events around every GEMM
    #    launch on its stream (hx_trace_enable); the kernels are the ones the graph replays ------------
    trace_kind = hg._lib.HX_TRACE_SPLIT_GEMM if args.precision == 'split' else hg._lib.HX_TRACE_SIMT_GEMM
    hg._lib.trace_read(trace_kind, reset=True)
    hg._lib.trace_enable(True)
    for i in range(args.steps):
        flush.fill_(float(i))
        step(e_dev)
    torch.cuda.synchronize()
    hg._lib.trace_enable(False)
    k_launches, k_ms, k_cmacs = hg._lib.trace_read(trace_kind, reset=True)
    if dist:
        dist.barrier()
    clocks = sampler.stop()
    step_ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    total_ms = max_over_ranks(sum(step_ms), dist, dev)
    value = world * args.steps / (total_ms * 1e-3)
    ms_per_step = total_ms / args.steps
    gpu_launches = launches  # our kernels only (the L2 flush is a torch fill, not counted); graph replays count theirs

    # -- end to end through the public API with host buffers ------------------------------------------
    # Every step uploads its pupil field from pinned host memory and reads its image back.  The copies run on
    # their own streams, double-buffered, so step i+1's upload and step i-1's download overlap step i's
    # transforms (as a streaming user would run them); the timed region spans all three streams.  Unless
    # --no-graph, the chain runs as two hcipy_gb300.CapturedCall graphs of the public API, one per input
    # buffer, alternating: each upload lands in its graph's input, and a graph replays only after the download
    # of its previous image.
    e_host = torch.from_numpy(w['E'].astype(np.complex64)).pin_memory()
    img_host = [torch.empty(focal.size, dtype=img.dtype).pin_memory() for _ in range(2)]  # complex128 (split)
    e2e_steps = max(10, min(args.steps, 100))
    h2d, d2h = torch.cuda.Stream(), torch.cuda.Stream()
    e2e_graphs = None if args.no_graph else [hg.CapturedCall(step, e_dev) for _ in range(2)]
    d_in = [g.static_in[0] for g in e2e_graphs] if e2e_graphs else [torch.empty_like(e_dev) for _ in range(2)]
    in_ready = [torch.cuda.Event() for _ in range(2)]
    in_free = [torch.cuda.Event() for _ in range(2)]
    out_done = [torch.cuda.Event() for _ in range(2)]

    def e2e_run(n):
        used = [False, False]
        for i in range(n):
            b = i % 2
            if used[b]:
                h2d.wait_event(in_free[b])
            with torch.cuda.stream(h2d):
                d_in[b].copy_(e_host, non_blocking=True)
                in_ready[b].record(h2d)
            stream.wait_event(in_ready[b])
            if e2e_graphs:
                if used[b]:
                    stream.wait_event(out_done[b])  # the graph's output buffer is free again
                res = e2e_graphs[b](d_in[b])
            else:
                res = step(d_in[b])
            in_free[b].record(stream)
            used[b] = True
            d2h.wait_stream(stream)
            with torch.cuda.stream(d2h):
                if not e2e_graphs:
                    res.record_stream(d2h)
                img_host[b].copy_(res, non_blocking=True)
                out_done[b].record(d2h)
        stream.wait_stream(d2h)

    e2e_run(4)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    t0.record(stream)
    h2d.wait_event(t0)
    e2e_run(e2e_steps)
    t1.record(stream)
    t1.synchronize()
    e2e_ms = max_over_ranks(t0.elapsed_time(t1), dist, dev)
    e2e_value = world * e2e_steps / (e2e_ms * 1e-3)
    img_host = img_host[(e2e_steps - 1) % 2]

    if rank != 0:
        return

    # -- roofline of the dominant kernel (the complex GEMM: all launches of a step) -------------------
    peaks = {}
    try:
        with open(os.path.join(ROOT, 'MEASURED_PEAKS.json')) as f:
            peaks = json.load(f)
    except (OSError, ValueError):
        pass
    # achieved = algorithmic FLOP of the GEMM launches (8 per complex MAC, the reference's count) / their
    # summed CUDA-event durations, recorded live in the timed region on the launching stream.
    achieved_tflops = 8.0 * k_cmacs / (k_ms * 1e-3) / 1e12 if k_ms > 0 else 0.0
    if args.precision == 'split':
        peak = peaks.get('bf16_tflops', 1900.0)
        bound, peak_note = 'tensor', 'dense fp16/bf16 tensor rate, %s' % (
            'of measured (burst)' if 'bf16_tflops' in peaks else 'of fallback')
    else:
        props = torch.cuda.get_device_properties(dev)
        max_mhz = (clocks or {}).get('sm_max_mhz') or peaks.get('sm_max_mhz', 2070.0)
        peak = props.multi_processor_count * 128 * 2 * max_mhz * 1e6 / 1e12
        bound = 'fp32'
        peak_note = ('nominal FP32 CUDA-core rate %d SMs x 128 lanes x 2 FLOP x %.0f MHz; '
                     'MEASURED_PEAKS.json has no FP32 figure' % (props.multi_processor_count, max_mhz))
    traffic = None
    tpath = os.path.join(ROOT, 'profiles', 'traffic.json')
    if os.path.exists(tpath):
        with open(tpath) as f:
            traffic = json.load(f).get('lyot2048_%s' % args.precision)

    # -- accuracy against the float64 oracle -----------------------------------------------------------
    from oracle import optics
    chain64 = optics.LyotChain(oracle_grid(pupil), oracle_grid(fpm_grid), oracle_grid(focal), w['fpm'], w['stop'])
    ref_img = chain64(w['E'])
    peak_img = np.abs(chain64.image(w['aperture'].astype(np.complex128))).max()**2
    ni_max, ni_mean, ni_level = dark_hole_error(img.cpu().numpy(), ref_img, focal, peak_img)

    cpu = None
    if not args.no_cpu_baseline and world == 1:
        v, n, dt = cpu_port_time(w, np.complex64, args.cpu_seconds)
        cpu = {'value': v, 'unit': UNIT, 'cores': host_cores(), 'kind': 'port',
               'sample': '%d propagations of the same workload in %.1f s (numpy/OpenBLAS cgemm, complex64, '
                         'matrices precomputed)' % (n, dt)}

    line = {
        'metric': METRIC, 'value': value, 'unit': UNIT, 'n_gpus': world, 'steps': args.steps,
        'warmup': args.warmup, 'ms_per_step': ms_per_step, 'higher_is_better': True, 'scaling': 'weak',
        'vs_baseline': None, 'dtype': 'fp32' if args.precision == 'fp32' else 'fp16x3-split/fp32-acc',
        'data': 'synthetic (seeded Zernike 2-100 aberrations, 1 nm RMS)',
        'config': {'workload': 'lyot-coronagraph 2048^2 pupil -> 512^2 FPM grid -> 512^2 image (3 MFTs)',
                   'pupil': args.pupil, 'fpm_grid': int(fpm_grid.dims[0]), 'image': int(focal.dims[0]),
                   'batch': 1, 'precision': args.precision, 'field_dtype': 'complex64',
                   'tiles': ('autotuned during the warm-up (hx_autotune)' if not args.no_autotune
                             else 'built-in choice'),
                   'launch': 'CUDA graph of the step, replayed' if not args.no_graph else 'Python launches',
                   'l2': 'flushed between steps (256 MiB write outside the per-step events)',
                   'parallelism': 'replicas' if world > 1 else 'single-gpu'},
        'roofline': {'bound': bound, 'achieved': achieved_tflops, 'peak': peak, 'unit': 'TFLOP/s',
                     'frac': achieved_tflops / peak, 'traffic': traffic,
                     'kernel': 'cgemm_nn_simt<float>' if args.precision == 'fp32' else 'split_gemm_kernel (tcgen05)',
                     'launches_per_step': k_launches / args.steps, 'ms_per_launch': k_ms / max(k_launches, 1),
                     'kernel_share_of_step': k_ms / total_ms if total_ms > 0 else None,
                     'algorithmic': '%d complex MACs x 8 FLOP per propagation' % cmacs, 'peak_note': peak_note,
                     'tensor_flop_per_algorithmic_flop': 8 if args.precision == 'split' else None},
        'e2e': {'value': e2e_value, 'unit': UNIT, 'h2d_bytes_per_step': int(e_host.numel() * 8),
                'd2h_bytes_per_step': int(img_host.numel() * img_host.element_size()),
                'launch': ('two alternating hcipy_gb300.CapturedCall graphs of the chain' if e2e_graphs
                           else 'Python launches of the chain'),
                'e2e_image_equals_device_image': bool(np.array_equal(img_host.numpy(), img.cpu().numpy()))},
        'gpu_launches': int(gpu_launches),
        'clocks': clocks,
        'wall_s_timed': wall,
    }
    accuracy = {'ni_err_max': ni_max, 'ni_err_mean': ni_mean, 'ni_err_bound': NI_BOUND,
                'meets_bound': bool(ni_max <= NI_BOUND), 'dark_hole_mean_ni': ni_level,
                'region': '3-15 lambda/D', 'against': 'float64 oracle chain on the same input'}
    if cpu is not None:
        line['cpu_baseline'] = cpu
    line['config']['autotuned_tiles'] = [
        {'shape': list(shape), 'best': list(c[0]), 'measured': [list(x) for x in c]}
        for shape, c in hg._lib.autotune_table()]
    if args.lyot_batch > 0:
        line['lyot_batched'] = run_lyot_batched(args, dev, ref_img, peak_img)
    if args.grad_steps > 0:
        line['grad_steps'] = run_grad(args, dev)
    if not args.no_atmosphere:
        line['atmosphere'] = run_atmosphere(args, dev, peaks)
    if args.broadband_frames > 0:
        line['broadband_turbulence'] = run_broadband(args, dev, peaks)
    if not args.no_small:
        line['dm_probes'] = run_dm_probes(args, dev)
        line['efc'] = run_efc(args, dev)
        line['fraunhofer_256'] = run_small_fraunhofer(args, dev, peaks)
        line['modulated_pyramid_256'] = run_modulated_pyramid(args, dev)
        line['vortex_256'] = run_vortex(args, dev)
        line['fft_family_1024'] = run_fft_family(args, dev, peaks)
    # The accuracy conditions of the metric and the side-by-side rates come last, so that a reader who keeps only
    # the end of the line (or of stderr, where the same summary is printed) still has them.
    line['accuracy'] = accuracy
    line['summary'] = headline_summary(line)
    print('summary: ' + json.dumps(line['summary']), file=sys.stderr, flush=True)
    print(json.dumps(line), flush=True)


def headline_summary(line):
    """The accuracy figures of every leg and the split/FP32 ratios in one short object."""
    s = {'propagations_per_s': line['value'], 'e2e_propagations_per_s': line['e2e']['value'],
         'ni_err_max': line['accuracy']['ni_err_max'], 'ni_err_bound': NI_BOUND,
         'meets_bound': line['accuracy']['meets_bound']}
    lb = line.get('lyot_batched')
    if lb:
        s['fp32_one_field_propagations_per_s'] = lb['fp32']['propagations_per_s_one_field']
        s['split_one_field_propagations_per_s'] = lb['split']['propagations_per_s_one_field']
        s['split_over_fp32_one_field'] = lb['split_over_fp32_one_field']
        s['split_over_fp32_batch%d' % lb['batch']] = lb['split_over_fp32']
        s['fp32_ni_err_max'] = lb['fp32'].get('ni_err_max_field0')
    gs = line.get('grad_steps')
    if gs:
        s['grad_steps_per_s'] = gs['value']
        s['grad_rel_err_max'] = gs['accuracy']['grad_rel_l2_err_max']
    bb = line.get('broadband_turbulence')
    if bb:
        s['broadband_frames_per_s_split'] = bb['split']['frames_per_s']
        s['broadband_centre_ni_err_max_split'] = bb['split'].get('ni_err_max_centre')
        s['broadband_centre_ni_err_max_fp32'] = bb['fp32'].get('ni_err_max_centre')
    return s


def main():
    args = parse_args()
    world = int(os.environ.get('WORLD_SIZE', '1'))
    rank = int(os.environ.get('RANK', '0'))
    dist = None
    if args.impl == 'reference':
        return run_reference(args, rank, world)
    if world > 1:
        import torch
        import torch.distributed as tdist
        torch.cuda.set_device(int(os.environ.get('LOCAL_RANK', 0)))
        tdist.init_process_group('nccl')
        dist = tdist
    try:
        run_ours(args, rank, world, dist)
    finally:
        if dist is not None:
            dist.destroy_process_group()


if __name__ == '__main__':
    main()
