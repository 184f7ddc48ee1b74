#!/usr/bin/env python
"""
Benchmark of the per-step Tersoff force path on GB300.

Workload (the configuration the headline metric is quoted on): Si block of
1,048,576 atoms at 2.33 g/cm^3 in a cubic periodic box, diamond sites with
Gaussian sigma = 0.25 A (seeded; atomistica_gb300.structures.
tersoff_si_amorphous).  One step = one energy_and_forces call: full
neighbour-list rebuild (positions are marked changed every step, as on the
reference's ASE path with a zero Verlet shell) + energy, forces and virial.

  value   atom-evals/s of the FP32-mixed form, inputs resident in HBM,
          CUDA events on the launching stream, L2 flushed between steps
          (256 MB write, outside the timed events); the FP64 drop-in is
          timed the same way and reported beside it.
  e2e     the same metric through the public API with pinned HOST buffers:
          per step the position upload and the force/energy/virial download
          are timed (forces written, as the reference's call without a forces
          argument returns a fresh array).
  roofline  the dominant kernel (bond-order tile kernel, mixed form):
          algorithmic FP32/FP64 flops per launch / kernel time against the
          FP32 and FP64 FMA peaks measured in this run.
  cpu_baseline  the C++ FP64 oracle (the reference algorithm restated;
          reference binary unavailable: no Fortran compiler) with OpenMP on
          all host cores, full workload, median of 3 calls.

python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
Under torchrun (N > 1) every rank evaluates its own replica (no exchange).
"""

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Tersoff atom-evals/s: FP32-mixed vs FP64 GPU at ≤1e-5 eV/Å force error"
UNIT = "atom-evals/s"

# Algorithmic flop model per directed bond and per triplet (+,-,*,/,sqrt and
# each exp/pow/cos/sin counted as one flop), counted from the reference's
# non-screened BOP code.  Both forms execute all of it: the FP64 drop-in on
# the FP64 pipe, the mixed form on the FP32 pipe (FP32 three-body terms,
# float-float geometry, pair terms and accumulation).
FLOPS_BOND = 150.0
FLOPS_TRIPLET = 165.0
# Compulsory DRAM bytes of one bond-order tile launch: per atom positions
# (32 B), element (4 B) and CSR offset (4 B); per directed bond the neighbour
# index and packed shift (8 B) in, the bond force G (24 B) out.
BYTES_ATOM = 40.0
BYTES_BOND = 32.0
# DRAM bytes (read + write) of one launch of the mixed tile kernel at this
# workload, from the ncu capture summarised in
# profiles/bop_tile_mx_tersoff_si_1048576.md (a past capture of the kernel
# named there, hot-bond threshold 1.2e-5 eV/A; not a measurement of this run).
TRAFFIC_MX = 75.59e6 + 49.54e6
# Alloy EAM flop model per list entry, counted from the reference's kernel
# (tabulated_alloy_eam.f90:423-627): the density pass (displacement 21,
# dot 5, sqrt, rho spline 11) and the force pass (phi spline f and df 14,
# 1/r, energy 2, rho' 8, force 10, f adds 6, virial 18), the latter being
# the algorithmic work of the pair kernel eam_pair.
EAM_FLOPS_DENSITY = 38.0
EAM_FLOPS_PAIR = 59.0


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--natoms", type=int, default=1048576)
    ap.add_argument("--seed", type=int, default=3)
    ap.add_argument("--cpu-runs", type=int, default=3)
    ap.add_argument("--config", default=None,
                    choices=["eam_cu_131072", "si_batch_2048", "si_fit_256"],
                    help="measure one of the other workloads alone and print its entry "
                         "(a short command for profiling it)")
    ap.add_argument("--skip-oracle", action="store_true",
                    help="skip the FP64 oracle error check and CPU baseline")
    ap.add_argument("--forms", default="fp64,mixed,fp64_graph,mixed_graph",
                    help="--config si_batch_2048: the forms to time (comma list); with "
                         "--skip-oracle only those run (a short command for a launch list)")
    return ap.parse_args()


def dist_info():
    from atomistica_gb300.distributed import dist_info as _di
    return _di()


class NvmlClockSampler:
    """SM clock and clock-event reasons sampled through NVML (read-only
    queries, libnvidia-ml via ctypes) about every millisecond by a thread, so
    that even a timed region of a few tens of milliseconds gets many samples.
    The device is matched to the CUDA device by UUID."""

    # nvmlClocksEventReasons bits
    REASONS = {0x4: "sw_power_cap", 0x8: "hw_slowdown", 0x20: "sw_thermal_slowdown",
               0x40: "hw_thermal_slowdown", 0x80: "hw_power_brake_slowdown"}

    def __init__(self, cuda_index):
        import ctypes
        import torch
        self.ct = ctypes
        self.nv = ctypes.CDLL("libnvidia-ml.so.1")
        if self.nv.nvmlInit_v2() != 0:
            raise RuntimeError("nvmlInit failed")
        self.h = ctypes.c_void_p()
        uuid = str(getattr(torch.cuda.get_device_properties(cuda_index), "uuid", ""))
        ok = False
        if uuid:
            u = uuid if uuid.startswith("GPU-") else "GPU-" + uuid
            ok = self.nv.nvmlDeviceGetHandleByUUID(u.encode(), ctypes.byref(self.h)) == 0
        if not ok:
            idx = os.environ.get("CUDA_VISIBLE_DEVICES", str(cuda_index)).split(",")[cuda_index]
            if self.nv.nvmlDeviceGetHandleByIndex_v2(int(idx), ctypes.byref(self.h)) != 0:
                raise RuntimeError("no NVML handle for the CUDA device")
        fn = getattr(self.nv, "nvmlDeviceGetCurrentClocksEventReasons", None)
        self.reasons_fn = fn or self.nv.nvmlDeviceGetCurrentClocksThrottleReasons
        mx = ctypes.c_uint()
        self.sm_max = float(mx.value) if self.nv.nvmlDeviceGetMaxClockInfo(
            self.h, 1, ctypes.byref(mx)) == 0 else None
        self.samples, self.reason_bits = [], 0
        self.thread, self.running = None, False

    def _loop(self):
        ct = self.ct
        clk, rs = ct.c_uint(), ct.c_ulonglong()
        while self.running:
            if self.nv.nvmlDeviceGetClockInfo(self.h, 1, ct.byref(clk)) == 0:  # NVML_CLOCK_SM
                self.samples.append(float(clk.value))
            if self.reasons_fn(self.h, ct.byref(rs)) == 0:
                self.reason_bits |= rs.value
            time.sleep(0.001)

    def start(self):
        import threading
        self._swi = sys.getswitchinterval()
        sys.setswitchinterval(0.0005)
        self.running = True
        self.thread = threading.Thread(target=self._loop, daemon=True)
        self.thread.start()

    def stop(self):
        self.running = False
        self.thread.join()
        sys.setswitchinterval(self._swi)
        reasons = sorted(n for b, n in self.REASONS.items() if self.reason_bits & b)
        sm = self.samples
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": self.sm_max,
                "sm_mhz_min": min(sm) if sm else None, "reasons": reasons, "samples": len(sm),
                "source": "NVML, ~1 ms sampling thread during the timed region"}


def clock_sampler(cuda_index):
    """NVML sampler, else the nvidia-smi one."""
    try:
        return NvmlClockSampler(cuda_index)
    except Exception:
        return ClockSampler(cuda_index)


class ClockSampler:
    """nvidia-smi clock / throttle-reason sampling during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.flush()
        self.f.seek(0)
        rows = [r.split(",") for r in self.f.read().splitlines() if r.strip()]
        os.unlink(self.f.name)
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            r = [x.strip() for x in r]
            if len(r) < 9:
                continue
            try:
                sm.append(float(r[1]))
                smax = float(r[2])
            except ValueError:
                continue
            for n, v in zip(names, r[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def flop_model(z):
    """Algorithmic flops and compulsory bytes of one bond-order evaluation."""
    import numpy as np
    z = np.asarray(z, dtype=np.float64)
    nb = float(z.sum())
    nt = float((z * (z - 1)).sum())
    return {"bonds": nb, "triplets": nt, "flops": FLOPS_BOND * nb + FLOPS_TRIPLET * nt,
            "bytes": BYTES_ATOM * len(z) + BYTES_BOND * nb}


def cpu_baseline(structure, params, runs, nthreads=None):
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle  # CPU baseline leg: the reference algorithm on the host cores
    oracle.build()
    nthreads = nthreads or oracle.max_threads()
    oracle.bop_compute("tersoff", params, structure, nthreads=nthreads)
    ts = []
    for _ in range(runs):
        t0 = time.perf_counter()
        oracle.bop_compute("tersoff", params, structure, nthreads=nthreads)
        ts.append(time.perf_counter() - t0)
    t = statistics.median(ts)
    return {"value": len(structure) / t, "unit": UNIT, "cores": nthreads, "kind": "port",
            "sample": "full %d-atom workload incl. neighbour build, median of %d calls "
                      "(C++ FP64 restatement of the reference algorithm, OpenMP, %d "
                      "thread%s)" % (len(structure), runs, nthreads, "" if nthreads == 1 else "s"),
            "seconds_per_call": t}


def _gpu_step_ms(pot, p, nl, d_pos, d_f, steps=20):
    """Mean device time (ms) of set_positions + energy_and_forces (forces
    written into d_f, as the reference's call without a forces argument
    returns a fresh array)."""
    import torch
    for _ in range(3):
        p.set_positions(d_pos)
        pot.energy_and_forces(p, nl, forces=d_f, accumulate=False)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(steps):
        p.set_positions(d_pos)
        pot.energy_and_forces(p, nl, forces=d_f, accumulate=False)
    e1.record()
    torch.cuda.synchronize()
    # whether the timed steps were graph replays: one more step with the
    # same arguments (the flag of a call is only visible after it)
    p.set_positions(d_pos)
    pot.energy_and_forces(p, nl, forces=d_f, accumulate=False)
    _gpu_step_ms.replayed = pot.last_replayed()
    return e0.elapsed_time(e1) / steps


def other_configs(dev, oracle):
    """The 4096-atom Tersoff crystal (FP64 and mixed) and the 131,072-atom
    alloy-EAM Cu block (FP64): GPU atom-evals/s through the public API with
    device-resident inputs (default stream, no L2 flush: both fit in L2),
    the oracle on all host cores, and the GPU-oracle deviations."""
    import numpy as np
    import torch
    from atomistica_gb300 import io as gio, native, parameters, structures
    out = {}
    nth = oracle.max_threads()

    def cpu_time(fn, runs=5):
        fn()
        ts = []
        for _ in range(runs):
            t0 = time.perf_counter()
            fn()
            ts.append(time.perf_counter() - t0)
        return statistics.median(ts)

    s = structures.tersoff_si_4096(seed=1)
    params = parameters.Tersoff_PRB_39_5566_Si_C
    ref = oracle.bop_compute("tersoff", params, s, nthreads=nth)
    t_cpu = cpu_time(lambda: oracle.bop_compute("tersoff", params, s, nthreads=nth))
    p = native.from_atoms(s)
    nl = native.Neighbors(100)
    d_pos = torch.tensor(s.positions, dtype=torch.float64, device=dev)
    d_f = torch.zeros((len(s), 3), dtype=torch.float64, device=dev)
    entry = {"natoms": len(s), "unit": UNIT, "cpu_oracle": len(s) / t_cpu, "cpu_cores": nth}
    for name in ("fp64", "mixed", "fp64_graph", "mixed_graph"):
        # (*_graph: CUDA-graph replay of whole evaluations, own particles/list)
        pq, nq = (native.from_atoms(s), native.Neighbors(100)) if "graph" in name else (p, nl)
        pot = native.Tersoff(precision=name.split("_")[0])
        pot.bind_to(pq, nq)
        if "graph" in name:
            pot.set_graph(True)
        ms = _gpu_step_ms(pot, pq, nq, d_pos, d_f)
        replayed = _gpu_step_ms.replayed
        d_f.zero_()
        pq.set_positions(d_pos)
        e, _, w = pot.energy_and_forces(pq, nq, forces=d_f)
        f = d_f.cpu().numpy()
        entry[name] = {"value": len(s) / (ms * 1e-3), "ms_per_step": ms,
                       "max_abs_dF": float(np.max(np.abs(f - ref["f"]))),
                       "abs_dE_per_atom": abs(e - ref["epot"]) / len(s)}
        if "graph" in name:
            entry[name]["replayed"] = replayed
    out["tersoff_si_4096"] = entry
    out["tersoff_scr"] = screened_config(dev, oracle, nth, cpu_time)
    out["md_si_4096"] = md_config()
    out["bop_forms"] = bop_forms_config(dev, oracle, nth, cpu_time)

    out["eam_cu_131072"] = eam_config(dev, oracle, nth, cpu_time)
    out["si_batch_2048"] = batch_config(dev, oracle, nth)
    out["si_fit_256"] = fitting_config(oracle, nth)
    return out


def eam_config(dev, oracle, nth, cpu_time):
    """The 131,072-atom alloy-EAM Cu block (FP64; analytic tables on 10,000
    points): atom-evals/s per step including the list build, the oracle on
    all host cores, the deviations, and the pair kernel against the FP64
    FMA peak."""
    import numpy as np
    import torch
    from atomistica_gb300 import io as gio, native, structures
    s = structures.eam_cu_131072(seed=2)
    with tempfile.TemporaryDirectory() as td:
        fn = os.path.join(td, "cu.setfl")
        gio.cu_analytic_setfl(fn)
        eo = oracle.EAM(fn)
        ref = eo.compute_full(s, nthreads=nth)
        t_cpu = cpu_time(lambda: eo.compute_full(s, nthreads=nth))
        p = native.from_atoms(s)
        nl = native.Neighbors(100)
        pot = native.TabulatedAlloyEAM(fn)
        pot.bind_to(p, nl)
        d_pos = torch.tensor(s.positions, dtype=torch.float64, device=dev)
        d_f = torch.zeros((len(s), 3), dtype=torch.float64, device=dev)
        ms = _gpu_step_ms(pot, p, nl, d_pos, d_f)
        d_f.zero_()
        p.set_positions(d_pos)
        e, _, w = pot.energy_and_forces(p, nl, forces=d_f)
        f = d_f.cpu().numpy()
        # the pair kernel alone (CUDA events on the potential's stream)
        pair_ms = []
        for _ in range(10):
            p.set_positions(d_pos)
            pot.energy_and_forces(p, nl, forces=d_f)
            pair_ms.append(pot.last_timing()[3])
        pair_ms = statistics.median(pair_ms)
        n_entries = int(nl.get_list(p)[0][-1])
        # the same step replayed as a CUDA graph (own particles and list)
        pg = native.from_atoms(s)
        nlg = native.Neighbors(100)
        potg = native.TabulatedAlloyEAM(fn)
        potg.bind_to(pg, nlg)
        potg.set_graph(True)
        ms_g = _gpu_step_ms(potg, pg, nlg, d_pos, d_f)
        replayed_g = _gpu_step_ms.replayed
        d_f.zero_()
        pg.set_positions(d_pos)
        e_g, _, _ = potg.energy_and_forces(pg, nlg, forces=d_f)
        graph = {"value": len(s) / (ms_g * 1e-3), "ms_per_step": ms_g,
                 "replayed": replayed_g,
                 "equals_eager": bool(e_g == e and np.array_equal(d_f.cpu().numpy(), f))}
    from atomistica_gb300 import _lib
    fp64_peak = _peak(_lib.load(), True)
    eam_roof = {"bound": "fp64", "kernel": "eam_pair (force pass)", "kernel_ms": pair_ms,
                "list_entries": n_entries, "flops_per_entry": EAM_FLOPS_PAIR,
                "achieved": EAM_FLOPS_PAIR * n_entries / (pair_ms * 1e-3) * 1e-12,
                "peak": fp64_peak, "unit": "TFLOP/s",
                "peak_source": "FP64 FMA-chain microbenchmark in this run"}
    eam_roof["frac"] = eam_roof["achieved"] / fp64_peak
    return {"natoms": len(s), "unit": UNIT, "cpu_oracle": len(s) / t_cpu, "cpu_cores": nth,
            "fp64": {"value": len(s) / (ms * 1e-3), "ms_per_step": ms,
                     "max_abs_dF": float(np.max(np.abs(f - ref["f"]))),
                     "abs_dE_per_atom": abs(e - ref["epot"]) / len(s)},
            "fp64_graph": graph,
            "roofline": eam_roof}


def bop_forms_config(dev, oracle, nth, cpu_time):
    """The other members of the bond-order template and the funcfl EAM, each
    against the oracle on all host cores (device-resident inputs, public API):
    Brenner / BrennerScr (Erhart-Albe Si-C) on a rattled B3-SiC crystal of
    32,768 atoms, Juslin (W-C-H) on a random W-C-H packing of 8,192 atoms,
    Juslin / JuslinScr on a rattled bcc W crystal of 8,192 sites with C and H
    substituted, and TabulatedEAM (analytic funcfl Cu) on a 32,000-atom fcc
    block."""
    import numpy as np
    import torch
    from atomistica_gb300 import io as gio, native, parameters, structures

    def measure(pot, s, ref):
        p = native.from_atoms(s)
        nl = native.Neighbors(100)
        pot.bind_to(p, nl)
        d_pos = torch.tensor(s.positions, dtype=torch.float64, device=dev)
        d_f = torch.zeros((len(s), 3), dtype=torch.float64, device=dev)
        ms = _gpu_step_ms(pot, p, nl, d_pos, d_f, steps=10)
        d_f.zero_()
        p.set_positions(d_pos)
        e, _, w = pot.energy_and_forces(p, nl, forces=d_f)
        f = d_f.cpu().numpy()
        return {"value": len(s) / (ms * 1e-3), "ms_per_step": ms,
                "max_abs_dF": float(np.max(np.abs(f - ref["f"]))),
                "abs_dE_per_atom": abs(e - ref["epot"]) / len(s)}

    out = {}
    sic = structures.b3(("Si", "C"), 4.3596, (16, 16, 16))
    sic.positions += np.random.default_rng(11).uniform(-0.1, 0.1, sic.positions.shape)
    wch = structures.random_wch(8192, seed=12)
    # bcc W with 10 % C and 5 % H on its sites (screened form: its kernel keeps
    # at most 32 bonds per atom after screening, which the dense random
    # packing exceeds under the front-end's weakly screening table)
    wcl = structures.bcc("W", 3.165, (16, 16, 16))
    rng = np.random.default_rng(14)
    u = rng.random(len(wcl))
    wcl.numbers[u < 0.15] = 6
    wcl.numbers[u < 0.05] = 1
    wcl.positions += rng.uniform(-0.1, 0.1, wcl.positions.shape)
    for name, s, kind, cls, params in (
            ("brenner_sic_32768", sic, "brenner", native.Brenner,
             parameters.Erhart_PRB_71_035211_SiC),
            ("brenner_scr_sic_32768", sic, "brenner_scr", native.BrennerScr,
             parameters.Erhart_PRB_71_035211_SiC__Scr),
            ("juslin_wch_8192", wch, "juslin", native.Juslin,
             parameters.Juslin_JAP_98_123520_WCH),
            ("juslin_wch_bcc_8192", wcl, "juslin", native.Juslin,
             parameters.Juslin_JAP_98_123520_WCH),
            ("juslin_scr_wch_bcc_8192", wcl, "juslin_scr", native.JuslinScr,
             parameters.Juslin_JAP_98_123520_WCH__Scr)):
        ref = oracle.bop_compute(kind, params, s, nthreads=nth)
        t_cpu = cpu_time(lambda: oracle.bop_compute(kind, params, s, nthreads=nth), runs=3)
        entry = {"natoms": len(s), "unit": UNIT, "cpu_oracle": len(s) / t_cpu,
                 "cpu_cores": nth}
        for prec in ("fp64",) if kind.endswith("_scr") else ("fp64", "mixed"):
            entry[prec] = measure(cls(precision=prec, **params), s, ref)
        out[name] = entry
    cu = structures.fcc("Cu", 3.615, (20, 20, 20))
    cu.positions += np.random.default_rng(13).normal(0.0, 0.05, cu.positions.shape)
    with tempfile.TemporaryDirectory() as td:
        fn = gio.cu_analytic_funcfl(os.path.join(td, "cu.eam"))
        fo = oracle.FuncflEAM(fn)
        ref = fo.compute(cu, nthreads=nth)
        t_cpu = cpu_time(lambda: fo.compute(cu, nthreads=nth), runs=3)
        out["funcfl_cu_32000"] = {"natoms": len(cu), "unit": UNIT, "cpu_oracle": len(cu) / t_cpu,
                                  "cpu_cores": nth,
                                  "fp64": measure(native.TabulatedEAM(fn), cu, ref)}
    return out


def md_config():
    """Velocity-Verlet MD of the 4096-atom Si crystal (a batch of one,
    Tersoff, dt = 1 fs): wall time per step of 200 steps, eager (list size and
    tile plan read back every step) and replayed as one CUDA graph per step."""
    import numpy as np
    from atomistica_gb300 import native, structures
    s = structures.tersoff_si_4096(seed=1)
    rng = np.random.default_rng(9)
    v = rng.normal(0.0, 0.02, (len(s), 3))
    m = np.full(len(s), 28.0855)
    out = {"natoms": len(s), "unit": "steps/s", "dt": 0.1, "mass_amu": 28.0855}
    for prec in ("fp64", "mixed"):
        pot = native.Tersoff(precision=prec)
        for graph in (False, True):
            b = native.Batch([s])
            b.set_options(graph=graph)
            b.md_set_state(v, m)
            b.md_run(pot, 0.1, 5)  # warm-up (and the capture)
            t0 = time.perf_counter()
            b.md_run(pot, 0.1, 200)
            t = (time.perf_counter() - t0) / 200
            out["%s_%s" % (prec, "graph" if graph else "eager")] = {
                "value": 1.0 / t, "ms_per_step": 1e3 * t,
                "atom_steps_per_s": len(s) / t, "replayed": b.last_info()["replayed"]}
    return out


def screened_config(dev, oracle, nth, cpu_time):
    """TersoffScr (FP64) on the 4096-atom Si crystal and on 4096 atoms of
    random carbon at 3.0 g/cm^3 (partially screened bonds everywhere): GPU
    atom-evals/s through the public API with device-resident inputs against
    the oracle on all host cores."""
    import numpy as np
    import torch
    from atomistica_gb300 import native, parameters, structures
    params = parameters.Tersoff_PRB_39_5566_Si_C__Scr
    out = {}
    for name, s in (("si_4096", structures.tersoff_si_4096(seed=1)),
                    ("aC_4096", structures.amorphous_carbon(4096, seed=7))):
        ref = oracle.bop_compute("tersoff_scr", params, s, nthreads=nth)
        t_cpu = cpu_time(lambda: oracle.bop_compute("tersoff_scr", params, s, nthreads=nth),
                         runs=3)
        p = native.from_atoms(s)
        nl = native.Neighbors(100)
        pot = native.TersoffScr()
        pot.bind_to(p, nl)
        d_pos = torch.tensor(s.positions, dtype=torch.float64, device=dev)
        d_f = torch.zeros((len(s), 3), dtype=torch.float64, device=dev)
        ms = _gpu_step_ms(pot, p, nl, d_pos, d_f, steps=5)
        d_f.zero_()
        p.set_positions(d_pos)
        e, _, w = pot.energy_and_forces(p, nl, forces=d_f)
        f = d_f.cpu().numpy()
        out[name] = {"natoms": len(s), "unit": UNIT, "cpu_oracle": len(s) / t_cpu,
                     "cpu_cores": nth, "neighbours_per_atom": pot.last_stats()[0] / len(s),
                     "fp64": {"value": len(s) / (ms * 1e-3), "ms_per_step": ms,
                              "kernel_ms": pot.last_timing()[3],
                              "max_abs_dF": float(np.max(np.abs(f - ref["f"]))),
                              "abs_dE_per_atom": abs(e - ref["epot"]) / len(s)}}
    return out


def batch_config(dev, oracle, nth, forms=("fp64", "mixed", "fp64_graph", "mixed_graph"),
                 check=True):
    """2048 triclinic Si structures, N ~ U{8..512}, in one batched evaluation
    (FP64 and mixed) against the same structures evaluated one call each on
    the GPU and by the oracle on all host cores."""
    import numpy as np
    import torch
    from atomistica_gb300 import native, parameters, structures
    t0 = time.perf_counter()
    structs = structures.si_batch(2048, seed=4)
    t_gen = time.perf_counter() - t0
    nat = sum(len(q) for q in structs)
    params = parameters.Tersoff_PRB_39_5566_Si_C
    r = torch.tensor(np.concatenate([q.positions for q in structs]), dtype=torch.float64,
                     device=dev)
    f = torch.zeros((nat, 3), dtype=torch.float64, device=dev)
    entry = {"nstruct": len(structs), "natoms": nat, "unit": UNIT,
             "generation_s": t_gen, "sample": "all 2048 structures"}
    refs = [oracle.bop_compute("tersoff", params, q, nthreads=nth) for q in structs] \
        if check else None
    # eager (list build and tile plan read back to the host each step) and
    # CUDA-graph replay of the whole step with autotuned tiles
    for name in forms:
        prec = name.split("_")[0]
        graph = name.endswith("_graph")
        b = native.Batch(structs)
        b.set_options(graph=graph, autotune=graph)
        pot = native.Tersoff(precision=prec)
        for _ in range(3):
            f.zero_()
            b.set_positions(r)
            b.energy_and_forces(pot, forces=f)
        torch.cuda.synchronize()
        steps = 10
        t0 = time.perf_counter()
        for _ in range(steps):
            f.zero_()
            b.set_positions(r)
            e, _, w = b.energy_and_forces(pot, forces=f)
        torch.cuda.synchronize()
        t = (time.perf_counter() - t0) / steps
        info = b.last_info()
        entry[name] = {"value": nat / t, "ms_per_step": 1e3 * t, "tile_bonds": info["tile_bonds"],
                       "replayed": info["replayed"], "graph_kernels": info["graph_kernels"]}
        if check:
            fh = f.cpu().numpy()
            eh = e.cpu().numpy()
            off = b.offsets
            entry[name]["max_abs_dF"] = max(
                float(np.max(np.abs(fh[off[q]:off[q + 1]] - refs[q]["f"])))
                for q in range(len(structs)))
            entry[name]["max_abs_dE_per_atom"] = max(
                abs(eh[q] - refs[q]["epot"]) / len(structs[q]) for q in range(len(structs)))
    if not check:
        return entry
    # the same structures one call each (particles + list + potential per structure)
    pot = native.Tersoff(precision="fp64")
    objs = []
    for q in structs:
        p = native.from_atoms(q)
        nl = native.Neighbors(100)
        pot.bind_to(p, nl)
        objs.append((p, nl, torch.tensor(q.positions, dtype=torch.float64, device=dev),
                     torch.zeros((len(q), 3), dtype=torch.float64, device=dev)))
    for p, nl, rq, fq in objs:
        pot.bind_to(p, nl)
        pot.energy_and_forces(p, nl, forces=fq)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for p, nl, rq, fq in objs:
        pot.bind_to(p, nl)
        p.set_positions(rq)
        pot.energy_and_forces(p, nl, forces=fq)
    torch.cuda.synchronize()
    entry["fp64_one_call_per_structure"] = {"value": nat / (time.perf_counter() - t0)}
    t0 = time.perf_counter()
    for q in structs:
        oracle.bop_compute("tersoff", params, q, nthreads=nth)
    entry["cpu_oracle"] = nat / (time.perf_counter() - t0)
    entry["cpu_cores"] = nth
    return entry


def fitting_config(oracle, nth):
    """Tersoff fitting loss over 256 diamond Si supercells (64-216 atoms):
    one forward + backward (loss gradient w.r.t. the 14 parameters and the
    positions: 1 evaluation + 1 adjoint pass, which gives the parameter
    gradient and the Hessian-vector product together), its agreement with
    central differences, and one energy+forces evaluation of the set by the
    oracle on the host cores."""
    import numpy as np
    import torch
    from atomistica_gb300 import fitting, structures
    structs = structures.si_fit_set(256, seed=5)
    nat = sum(len(q) for q in structs)
    theta, m = fitting.single_element_parameters()
    rng = np.random.default_rng(5)
    theta_t = theta * (1.0 + rng.uniform(-0.02, 0.02, size=14))
    tb = fitting.TersoffBatch(structs, m=m)
    r0 = np.concatenate([q.positions for q in structs])
    tb.set_positions(r0)
    et, _, ft, _ = tb.evaluate(theta_t)
    E_t, F_t = torch.tensor(et), torch.tensor(ft)

    def loss_grad():
        th = torch.tensor(theta, requires_grad=True)
        r = torch.tensor(r0, requires_grad=True)
        E, F = fitting.EnergyForces.apply(th, r, tb)
        loss = fitting.fitting_loss(E, F, tb.nat, E_t, F_t)
        loss.backward()
        return loss.item(), th.grad.numpy().copy()

    loss_grad()
    ts = []
    for _ in range(3):
        t0 = time.perf_counter()
        loss, g = loss_grad()
        ts.append(time.perf_counter() - t0)
    rel = []
    with torch.no_grad():
        for k in range(14):
            h = 1e-6 * abs(theta[k]) if theta[k] != 0 else 1e-6
            u = np.zeros(14)
            u[k] = h
            lv = []
            for sgn in (1.0, -1.0):
                E, F = fitting.EnergyForces.apply(torch.tensor(theta + sgn * u),
                                                  torch.tensor(r0), tb)
                lv.append(fitting.fitting_loss(E, F, tb.nat, E_t, F_t).item())
            fd = (lv[0] - lv[1]) / (2 * h)
            rel.append(abs(g[k] - fd) / max(abs(g[k]), abs(fd), 1e-300))
    params = fitting.parameter_dict(theta, m)
    t0 = time.perf_counter()
    for q in structs:
        oracle.bop("tersoff", params, q, per_at=False, nthreads=nth)
    t_cpu = time.perf_counter() - t0
    return {"nstruct": len(structs), "natoms": nat,
            "forward_backward_s": statistics.median(ts), "loss": loss,
            "grad_vs_central_differences_max_rel": max(rel),
            "cpu_oracle_one_evaluation_s": t_cpu, "cpu_cores": nth,
            "note": "central differences need 29 evaluations of the set"}


def run_reference(args):
    ws, rank, _ = dist_info()
    if rank != 0:
        return
    from atomistica_gb300 import parameters, structures
    s = structures.tersoff_si_amorphous(args.natoms, seed=args.seed)
    params = parameters.Tersoff_PRB_39_5566_Si_C
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    oracle.build()
    nthreads = oracle.max_threads()
    for _ in range(max(args.warmup, 1)):
        oracle.bop_compute("tersoff", params, s, nthreads=nthreads)
    ts = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        oracle.bop_compute("tersoff", params, s, nthreads=nthreads)
        ts.append(time.perf_counter() - t0)
    total = sum(ts)
    value = len(s) * args.steps / total
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "fp64",
        "data": "synthetic (seeded)",
        "config": {"workload": "tersoff_si_amorphous_%d" % len(s), "natoms": len(s),
                   "seed": args.seed, "density_gcc": 2.33, "sigma_A": 0.25},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": nthreads, "kind": "port",
                         "sample": "full workload per step incl. neighbour build (C++ FP64 "
                                   "restatement of the reference algorithm, OpenMP; reference "
                                   "binary unavailable: no Fortran compiler)"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_ours(args):
    import numpy as np
    import torch
    ws, rank, local = dist_info()
    if ws > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    else:
        torch.cuda.set_device(0)
    dev = torch.device("cuda", torch.cuda.current_device())

    from atomistica_gb300 import _lib, native, parameters, structures
    from atomistica_gb300 import build as gbuild
    gbuild.build()
    L = _lib.load()
    params = parameters.Tersoff_PRB_39_5566_Si_C
    s = structures.tersoff_si_amorphous(args.natoms, seed=args.seed)
    nat = len(s)

    stream = torch.cuda.Stream(device=dev)
    p = native.from_atoms(s)
    p.set_stream(stream.cuda_stream)
    nl = native.Neighbors(100)
    pots = {}
    for prec in ("mixed", "fp64"):
        pot = native.Tersoff(precision=prec)
        pot.set_stream(stream.cuda_stream)
        pot.bind_to(p, nl)
        pots[prec] = pot
    # the mixed form with CUDA-graph replay of whole evaluations
    # (gb_potential_set_graph), on its own particles and list
    pg = native.from_atoms(s)
    pg.set_stream(stream.cuda_stream)
    nlg = native.Neighbors(100)
    pots["mixed_graph"] = native.Tersoff(precision="mixed")
    pots["mixed_graph"].set_stream(stream.cuda_stream)
    pots["mixed_graph"].bind_to(pg, nlg)
    pots["mixed_graph"].set_graph(True)
    where = {"mixed": (p, nl), "fp64": (p, nl), "mixed_graph": (pg, nlg)}

    d_pos = torch.tensor(s.positions, dtype=torch.float64, device=dev)
    d_f = torch.zeros((nat, 3), dtype=torch.float64, device=dev)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=dev)  # 256 MB > L2

    def step(pot):
        pp, nn = next(where[k] for k, v in pots.items() if v is pot)
        pp.set_positions(d_pos)   # marks positions changed -> full neighbour rebuild
        # forces written (every atom), as the reference's call without a
        # forces argument returns a fresh array
        return pot.energy_and_forces(pp, nn, forces=d_f, accumulate=False)

    def timed(pot, k, sampler=None):
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
              for _ in range(k)]
        parts = []
        if ws > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()
        n0 = L.gb_kernel_launches()
        if sampler:
            sampler.start()
        replayed = 0
        for q in range(k):
            with torch.cuda.stream(stream):
                flush.zero_()
                ev[q][0].record(stream)
            step(pot)
            with torch.cuda.stream(stream):
                ev[q][1].record(stream)
            parts.append(pot.last_timing())
            replayed += pot.last_replayed()
        timed.replayed = replayed
        torch.cuda.synchronize()
        clocks = sampler.stop() if sampler else None
        launches = L.gb_kernel_launches() - n0
        if ws > 1:
            torch.distributed.barrier()
        ms = [a.elapsed_time(b) for a, b in ev]
        return ms, parts, launches, clocks

    for prec in ("fp64", "mixed", "mixed_graph"):
        for _ in range(max(args.warmup, 3)):
            step(pots[prec])
    torch.cuda.synchronize()

    ms64, parts64, _, _ = timed(pots["fp64"], args.steps)
    msmx, partsmx, launches_mx, _ = timed(pots["mixed"], args.steps)
    sampler = clock_sampler(torch.cuda.current_device())
    msg, _, launches, clocks = timed(pots["mixed_graph"], args.steps, sampler)
    replayed_g = timed.replayed

    from atomistica_gb300.distributed import max_over_ranks as tmax

    t_mx = tmax(sum(msmx) / 1e3)
    t_64 = tmax(sum(ms64) / 1e3)
    t_g = tmax(sum(msg) / 1e3)
    value = ws * nat * args.steps / t_g
    value_mx = ws * nat * args.steps / t_mx
    value64 = ws * nat * args.steps / t_64
    nl_mx = statistics.mean(q[0] for q in partsmx)
    kern_mx = statistics.mean(q[3] for q in partsmx)
    kern_64 = statistics.mean(q[3] for q in parts64)
    nl_64 = statistics.mean(q[0] for q in parts64)

    # Accuracy of both forms at the workload against each other and the oracle.
    res = {}
    for prec in ("fp64", "mixed", "mixed_graph"):
        e, f, w = step(pots[prec])
        res[prec] = (e, f.cpu().numpy().copy(), np.array(w))
    graph_equal = (res["mixed_graph"][0] == res["mixed"][0]
                   and np.array_equal(res["mixed_graph"][1], res["mixed"][1])
                   and np.array_equal(res["mixed_graph"][2], res["mixed"][2]))
    hot = pots["mixed"].last_stats()
    seed_np, _, _ = nl.get_list(p)
    fm = flop_model(np.diff(seed_np))

    # e2e through the public API: pinned host buffers, and the plain
    # (pageable) numpy arrays an ASE-style caller passes.
    pot = pots["mixed"]

    def e2e_rate(pos_np, f_np):
        for _ in range(2):
            p.set_positions(pos_np)
            pot.energy_and_forces(p, nl, forces=f_np, accumulate=False)
        if ws > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            p.set_positions(pos_np)
            pot.energy_and_forces(p, nl, forces=f_np, accumulate=False)
        torch.cuda.synchronize()
        t = tmax(time.perf_counter() - t0)
        return ws * nat * args.steps / t, 1e3 * t / args.steps

    pos_h = torch.empty((nat, 3), dtype=torch.float64).pin_memory()
    pos_h.copy_(torch.from_numpy(s.positions))
    f_h = torch.zeros((nat, 3), dtype=torch.float64).pin_memory()
    pot, (p, nl) = pots["mixed"], where["mixed"]
    e2e_mx_value, e2e_mx_ms = e2e_rate(pos_h.numpy(), f_h.numpy())
    pot, (p, nl) = pots["mixed_graph"], where["mixed_graph"]
    e2e_value, e2e_ms = e2e_rate(pos_h.numpy(), f_h.numpy())
    e2e_replayed = pot.last_replayed()
    pg_value, pg_ms = e2e_rate(np.array(s.positions, dtype=np.float64, order="C"),
                               np.zeros((nat, 3)))
    pot, (p, nl) = pots["mixed"], where["mixed"]
    e2e = {"value": e2e_value, "unit": UNIT, "ms_per_step": e2e_ms,
           "h2d_bytes_per_step": 24 * nat, "d2h_bytes_per_step": 24 * nat + 80,
           "api": "native.Particles.set_positions + Tersoff.energy_and_forces(accumulate="
                  "False) (C-ABI gb_particles_set_positions / "
                  "gb_potential_energy_and_forces_flags(GB_FORCES_SET)) on a potential with "
                  "set_graph(True) (gb_potential_set_graph: each step one CUDA-graph replay "
                  "of the whole evaluation, full neighbour rebuild included), pinned host "
                  "numpy buffers: positions up, forces written down",
           "replayed": bool(e2e_replayed),
           "pageable": {"value": pg_value, "unit": UNIT, "ms_per_step": pg_ms,
                        "buffers": "plain numpy arrays (pageable host memory), same calls"},
           "eager": {"value": e2e_mx_value, "unit": UNIT, "ms_per_step": e2e_mx_ms,
                     "api": "the same calls without the graph option (pinned buffers)"}}

    # Roofline of the dominant kernel (mixed bond-order tile kernel):
    # T_roof = max(flops / FP32 peak, bytes / HBM peak), frac = T_roof / t.
    p32 = _peak(L, 0)
    p64 = _peak(L, 1)
    hbm = _hbm_peak()
    t_k = kern_mx * 1e-3
    t_flop = fm["flops"] / (p32 * 1e12)
    t_byte = fm["bytes"] / (hbm * 1e9)
    roofline = {"bound": "fp32" if t_flop >= t_byte else "hbm",
                "achieved": fm["flops"] / t_k / 1e12, "peak": p32, "unit": "TFLOP/s",
                "frac": max(t_flop, t_byte) / t_k,
                "traffic": TRAFFIC_MX if nat == 1048576 else None,
                "traffic_source": "past ncu capture (dram__bytes_read.sum + dram__bytes_write.sum, one launch) "
                                  "(profiles/bop_tile_mx_tersoff_si_1048576.md)",
                "kernel": "bop_tile_mx<Tersoff> (mixed form)",
                "kernel_ms": kern_mx,
                "t_roof_ms": 1e3 * max(t_flop, t_byte),
                "bytes_per_launch": fm["bytes"], "hbm_gbs": hbm,
                "peak_source": "FP32/FP64 FMA-chain microbenchmark in this run (MEASURED_PEAKS.json "
                               "has no FP32/FP64 peak; no tensor cores on this path); HBM from "
                               "MEASURED_PEAKS.json",
                "fp32_peak_tflops": p32, "fp64_peak_tflops": p64,
                "fp64_form": {"kernel": "bop_tile<Tersoff, double>", "kernel_ms": kern_64,
                              "achieved_tflops": fm["flops"] / (kern_64 * 1e-3) / 1e12,
                              "frac_of_fp64_peak": fm["flops"] / (kern_64 * 1e-3)
                              / (p64 * 1e12)},
                "flop_model": {"per_bond": FLOPS_BOND, "per_triplet": FLOPS_TRIPLET,
                               "bonds": fm["bonds"], "triplets": fm["triplets"]}}

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * t_g / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "fp32 three-body terms + float-float (2 x fp32) geometry, pair terms, "
                 "bond order, accumulation; fp64 tile sums",
        "data": "synthetic (seeded)",
        "config": {"workload": "tersoff_si_amorphous_%d" % nat, "natoms": nat,
                   "seed": args.seed, "density_gcc": 2.33, "sigma_A": 0.25,
                   "potential": "Tersoff_PRB_39_5566_Si_C", "parallelism": "replicas" if ws > 1
                   else "single GPU", "l2": "flushed between steps (256 MB write outside the "
                                            "timed events)",
                   "step": "set_positions (D2D) + energy_and_forces (forces written, "
                           "accumulate=False) incl. full neighbour "
                           "rebuild, replayed as one CUDA graph (Tersoff.set_graph(True), "
                           "gb_potential_set_graph; results equal the eager path's bit for "
                           "bit, checked below)"},
        "fp64_dropin": {"value": value64, "unit": UNIT, "ms_per_step": 1e3 * t_64 / args.steps,
                        "neighbour_ms": nl_64, "kernel_ms": kern_64},
        "mixed_over_fp64": value_mx / value64,
        "replayed_steps": int(replayed_g),
        "graph_equals_eager": bool(graph_equal),
        "eager": {"value": value_mx, "unit": UNIT, "ms_per_step": 1e3 * t_mx / args.steps,
                  "gpu_launches": int(launches_mx), "neighbour_ms": nl_mx, "kernel_ms": kern_mx,
                  "value_without_neighbour_build":
                      ws * nat / ((1e3 * t_mx / args.steps - nl_mx) * 1e-3),
                  "api": "the same calls without the graph option (host synchronisations: "
                         "list sizes, final results)"},
        "mixed_accurate_path": {"bonds": hot[0], "recomputed": hot[1],
                                "fraction": hot[1] / max(hot[0], 1), "atoms_per_tile": hot[2]},
        "e2e": e2e,
        "roofline": roofline,
        "gpu_launches": int(launches),
        "clocks": clocks,
    }
    emx, fmx, wmx = res["mixed"]
    e64, f64, w64 = res["fp64"]
    line["accuracy"] = {"mixed_vs_fp64_gpu": {"max_abs_dF": float(np.max(np.abs(fmx - f64))),
                                              "abs_dE_per_atom": abs(emx - e64) / nat,
                                              "max_abs_dW": float(np.max(np.abs(wmx - w64)))}}
    if rank == 0 and not args.skip_oracle:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle  # the FP64 checker and the CPU baseline
        oracle.build()
        ref = oracle.bop_compute("tersoff", params, s, nthreads=oracle.max_threads())
        for prec, (e, f, w) in res.items():
            line["accuracy"][prec + "_vs_oracle"] = {
                "max_abs_dF": float(np.max(np.abs(f - ref["f"]))),
                "abs_dE_per_atom": abs(e - ref["epot"]) / nat,
                "max_abs_dW": float(np.max(np.abs(w - ref["wpot"])))}
        line["cpu_baseline"] = cpu_baseline(s, params, args.cpu_runs)
        line["cpu_baseline_1thread"] = cpu_baseline(s, params, 1, nthreads=1)
        line["other_configs"] = other_configs(dev, oracle)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if ws > 1:
        torch.distributed.destroy_process_group()


def _hbm_peak():
    """Measured HBM copy bandwidth (GB/s) from MEASURED_PEAKS.json, else the
    profiling fallback 6800 GB/s."""
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            return float(json.load(fh)["hbm_gbs"])
    except (OSError, KeyError, ValueError):
        return 6800.0


_peaks = {}


def _peak(L, fp64):
    import ctypes
    if fp64 not in _peaks:
        v = ctypes.c_double(0.0)
        _lib_check = L.gb_bench_fma_peak(int(fp64), ctypes.byref(v))
        if _lib_check != 0:
            raise RuntimeError("FMA peak microbenchmark failed")
        _peaks[fp64] = v.value
    return _peaks[fp64]


def run_config(args):
    """One of the other workloads alone (its JSON entry on one line)."""
    import torch
    torch.cuda.set_device(0)
    dev = torch.device("cuda", 0)
    from atomistica_gb300 import build as gbuild
    gbuild.build()
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle  # the checker and the CPU baseline
    nth = oracle.max_threads()

    def cpu_time(fn, runs=1):
        t0 = time.perf_counter()
        fn()
        return time.perf_counter() - t0

    if args.config == "eam_cu_131072":
        entry = eam_config(dev, oracle, nth, cpu_time)
    elif args.config == "si_batch_2048":
        entry = batch_config(dev, oracle, nth, tuple(args.forms.split(",")),
                             check=not args.skip_oracle)
    else:
        entry = fitting_config(oracle, nth)
    print(json.dumps({"config": args.config, **entry}))


def main():
    args = parse_args()
    if args.impl == "reference":
        run_reference(args)
    elif args.config:
        run_config(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
