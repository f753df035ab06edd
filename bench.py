"""Benchmark of the GB300 cook force path (one JSON line on rank 0).

A step is one MD step of the workload (linked-cell LJ + Ewald r-space sum,
classical Ewald k-space sum, leap-frog + SHAKE) with the coordinates resident
on the device.  The headline is the mixed-precision path (FP32 arithmetic,
FP64 accumulation); the plain FP64 path runs the same steps for the ratio.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

N > 1 runs under torchrun: independent replicas (the path does not shard),
one box per GPU, barrier + max-over-ranks time, value = total over ranks.
"""
import argparse
import json
import math
import os
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

METRIC = "ns/day & atom-steps/s, mixed vs plain FP64 GPU path at force RMS err ≤1e-5"
WORKLOAD = "spce32768"
FLOP_PER_PAIR = 45          # FP32 flops per in-cutoff (half) pair
FLOP_PER_KQ = 8             # flops per (k-vector, charge) per Ewald pass


def env_rank():
    return (int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)),
            int(os.environ.get("LOCAL_RANK", 0)))


# ------------------------------------------------------------------ clocks --

class ClockSampler:
    """nvidia-smi clocks/throttle reasons sampled every 200 ms (background)"""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = str(gpu_index)
        self.proc = None
        self.path = tempfile.mktemp(prefix="clocks_", suffix=".csv")

    def start(self):
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", self.gpu, "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "50"],
                stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
            return
        # the sampler is running once its first line is written: time after it
        t0 = time.time()
        while time.time() - t0 < 3.0:
            self.f.flush()
            if os.path.getsize(self.path) > 0:
                break
            time.sleep(0.02)

    def stop(self):
        out = {"sm_mhz": None, "sm_max_mhz": None, "reasons": []}
        if self.proc is None:
            return out
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            p = [x.strip() for x in line.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                mx.append(float(p[2]))
            except ValueError:
                continue
            for k, nm in enumerate(names):
                if p[5 + k].lower() == "active":
                    reasons.add(nm)
        os.unlink(self.path)
        if sm:
            out = {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(mx)),
                   "reasons": sorted(reasons), "samples": len(sm)}
        return out


# ------------------------------------------------------------ CPU baseline --

def cpu_md_steps(w, nsteps_max, budget_s, nthreads):
    """the oracle port (C, pthreads) on the host cores: MD steps of the
    workload (Drude systems: linear predictor + one SCF iteration per step)"""
    from oracle import oracle as O
    system = w["system"]
    ns = system.ns
    orc = O.Oracle(system, [w["L"]] * 3, w["cutoff"], w["alpha"], w["kappa"])
    r, r1 = w["r"].copy(), w["r1"].copy()
    t0 = time.perf_counter()
    done = 0
    prev = r[ns:].copy() if system.polar else None
    while done < nsteps_max:
        if system.polar:
            cur = r[ns:].copy()
            r = np.vstack([r[:ns], 2 * cur - prev])
            prev = cur
            f, _ = orc.forces(r, measure=False, nthreads=nthreads)
            r, f, _, _ = orc.selffield(r, f, 4.0 / 7.0)
            rs, r1s, it, _ = orc.shake_step(r[:ns], r1[:ns], f[:ns], w["h"], eps=1e-7, omega=0.6)
            r = np.vstack([rs, r[ns:]])
            r1 = np.vstack([r1s, r1[ns:]])
        else:
            f, _ = orc.forces(r, measure=False, nthreads=nthreads)
            r, r1, it, _ = orc.shake_step(r, r1, f, w["h"], eps=1e-7, omega=0.6)
        done += 1
        if time.perf_counter() - t0 > budget_s:
            break
    return done, time.perf_counter() - t0


def ns_per_day(h_ps, steps, seconds):
    return 86.4 * h_ps * steps / seconds


# ---------------------------------------------------------------- our arm --

def run_ours(args, rank, world, local):
    import torch
    import torch.distributed as dist
    import macsimus_gb300 as M
    from macsimus_gb300 import configs

    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    w = configs.workload(args.workload, seed=1000 + rank)
    if args.equilibrate > 0:
        w = configs.equilibrate(w, steps=args.equilibrate, h=0.001)
    system = w["system"]
    ns = system.ns
    stream = torch.cuda.current_stream()

    def barrier():
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()

    kw = dict(h=w["h"], epsc=1e-7, aspc_k=w["aspc_k"], scf_iter=w["scf_iter"], skin=args.skin,
              kspace_engine=args.kspace_engine or 0)
    # the autotuner picks the cell subdivision and the Ewald pass-1 split on
    # this configuration (untimed)
    tuned = {}
    if not args.no_autotune:
        best = M.autotune(system, [w["L"]] * 3, w["cutoff"], w["alpha"], w["kappa"], w["r"],
                          precision="mixed", **kw)
        tuned = dict(cells_per_cutoff=best["cells_per_cutoff"],
                     kspace_ctas_per_sm=best["kspace_ctas_per_sm"],
                     pair_variant=best["pair_variant"], kspace_serial=best["kspace_serial"])
    if args.pair_variant is not None:
        tuned["pair_variant"] = args.pair_variant
    if args.cells is not None:
        tuned["cells_per_cutoff"] = args.cells
    if args.kspace_serial is not None:
        tuned["kspace_serial"] = args.kspace_serial
    fp = M.ForcePath(system, [w["L"]] * 3, w["cutoff"], w["alpha"], w["kappa"], precision="mixed",
                     **kw, **tuned)
    fp.set_stream(stream.cuda_stream)
    # accuracy of the mixed path against the FP64 path on the same input
    f64 = M.ForcePath(system, [w["L"]] * 3, w["cutoff"], w["alpha"], w["kappa"],
                      precision="fp64", **kw)
    f64.set_stream(stream.cuda_stream)
    fm, em = fp.forces(w["r"], measure=True)
    fd, ed = f64.forces(w["r"], measure=True)
    force_err = float(np.sqrt(((fm - fd) ** 2).sum() / (fd ** 2).sum()))
    # the energies beside the forces: the k-space energy relative to itself
    # (the tensor-core passes accumulate in FP32 rounded toward zero), the
    # total potential energy relative to the Ewald energy scale |E_self|
    energy_err = {"ek_rel": (em["ek"] - ed["ek"]) / abs(ed["ek"]),
                  "epot_rel_eself": (em["el"] + em["lj"] - ed["el"] - ed["lj"]) / abs(ed["eself"]),
                  "lj_rel": (em["lj"] - ed["lj"]) / abs(ed["lj"])}

    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device="cuda")

    def timed_steps(path, k, warm, profile=False):
        path.md_set_state(w["r"], w["r1"])
        for _ in range(warm):
            path.md_steps(1, measure=False)
        barrier()
        path.profile(profile)
        path.profile_reset()
        launches = 0
        total_ms = 0.0
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        for _ in range(k):
            flush.fill_(1)          # L2 flushed between timed steps (outside the events)
            e0.record(stream)
            path.md_steps(1, measure=False)
            e1.record(stream)
            e1.synchronize()
            total_ms += e0.elapsed_time(e1)
            launches += path.launches
        barrier()
        prof = path.profile_read() if profile else {}
        path.profile(False)
        return total_ms, launches, prof

    gpu_index = local
    vis = os.environ.get("CUDA_VISIBLE_DEVICES")
    if vis:
        try:
            gpu_index = int(vis.split(",")[local])
        except ValueError:
            pass
    if not args.no_autotune and args.kspace_serial is None and fp.precision == "mixed":
        # the Ewald chain beside or after the r-space chain: the autotuner
        # times warm force evaluations, while the step runs as a graph after
        # an L2 flush and can rank the two the other way; a few untimed
        # steps of each decide
        best = None
        for ser in (0, 1):
            fp.set_overlap(not ser)
            ms_try, _, _ = timed_steps(fp, 10, 3)
            if best is None or ms_try < best[1]:
                best = (ser, ms_try)
        tuned["kspace_serial"] = best[0]
        fp.set_overlap(not best[0])
    clocks = ClockSampler(gpu_index)
    clocks.start()
    total_ms, launches, _ = timed_steps(fp, args.steps, args.warmup)
    clk = clocks.stop()
    # per-kernel times (roofline, shares) from a separate pass with the
    # k-space and r-space chains serialised, so that no kernel shares the GPU
    fp.set_overlap(False)
    _, _, prof = timed_steps(fp, min(args.steps, 20), 2, profile=True)
    fp.set_overlap(not tuned.get("kspace_serial", 0))
    t = torch.tensor([total_ms], dtype=torch.float64, device="cuda")
    if world > 1:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    total_ms = float(t.item())
    ms_step = total_ms / args.steps
    value = world * ns_per_day(w["h"], args.steps, total_ms * 1e-3)
    atom_steps = world * ns * args.steps / (total_ms * 1e-3)

    # plain FP64 path, same workload (fewer steps: it is ~2 orders slower)
    k64 = max(1, min(args.steps, args.fp64_steps))
    ms64, _, _ = timed_steps(f64, k64, 1)
    t = torch.tensor([ms64], dtype=torch.float64, device="cuda")
    if world > 1:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    value64 = world * ns_per_day(w["h"], k64, float(t.item()) * 1e-3)

    # end to end through the C ABI with pinned host buffers, as a host MD
    # loop that keeps the coordinates calls it: every step copies r, r1 in,
    # runs the step (forces without energies, as cook between measurement
    # cycles) and reads the new r, r1 back into the same pinned buffers
    rh = torch.from_numpy(w["r"].reshape(-1).copy()).pin_memory().numpy()
    r1h = torch.from_numpy(w["r1"].reshape(-1).copy()).pin_memory().numpy()
    ke2e = max(3, min(args.steps, 50))
    barrier()
    t0 = time.perf_counter()
    for _ in range(ke2e):
        fp.md_set_state(rh, r1h)
        fp.md_steps(1, measure=False)
        fp.md_get_state(out=(rh, r1h))
    barrier()
    e2e_s = time.perf_counter() - t0
    t = torch.tensor([e2e_s], dtype=torch.float64, device="cuda")
    if world > 1:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    e2e = world * ns_per_day(w["h"], ke2e, float(t.item()))

    # roofline of the dominant kernel (FP32 pipe: no tensor-core contraction here)
    peak = M.fp32_peak_tflops()
    nq = int((system.q != 0).sum()) + (int((system.qpol != 0).sum()) if system.polar else 0)
    V = w["L"] ** 3
    npairs = ns * (ns - 1) / 2 * (4.0 / 3.0 * math.pi * w["cutoff"] ** 3) / V
    algo = {"ewald_sk": FLOP_PER_KQ * fp.nkvec * nq, "ewald_kforce": FLOP_PER_KQ * fp.nkvec * nq,
            "pair_mixed": FLOP_PER_PAIR * npairs}
    # the kernel with the largest share among those with algorithmic work
    # (the small cell-list kernels of a small box are mostly launch gaps)
    work = {k: v for k, v in prof.items() if k in algo}
    top = max(work.items(), key=lambda kv: kv[1][0]) if work else ("none", (0, 1))
    name, (kms, kcnt) = top
    kavg = kms / max(kcnt, 1)
    achieved = algo.get(name, 0) / (kavg * 1e-3) / 1e12 if kavg > 0 else 0.0
    # the pair step's kernel: the group kernel (pair_variant 8), its half-shell
    # forms (9: lanes on the home sites, 10: lanes on the neighbours; with
    # Drude shells 10 runs 9) or the cell kernel
    if name == "pair_mixed" and tuned.get("pair_variant", 0) in (8, 9, 10):
        pv = tuned["pair_variant"]
        name = {8: "pair_group", 9: "pair_half", 10: "pair_half" if system.polar
                else "pair_half_t"}[pv]
        algo[name] = algo["pair_mixed"]
        achieved = algo[name] / (kavg * 1e-3) / 1e12 if kavg > 0 else 0.0
    traffic = None
    tpath = os.path.join(REPO, "profiles", "traffic_%s.json" % args.workload)
    if os.path.exists(tpath):
        traffic = json.load(open(tpath)).get(name)
    shares = {k: round(v[0] / max(sum(x[0] for x in prof.values()), 1e-30), 4)
              for k, v in prof.items()}

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        nth = os.cpu_count() or 1
        # a bounded sample: MD steps until about cpu_budget seconds of CPU work
        done, secs = cpu_md_steps(w, 10 ** 6, args.cpu_budget, nth)
        cpu = {"value": ns_per_day(w["h"], done, secs), "unit": "ns/day", "cores": nth,
               "kind": "port",
               "sample": "%d MD step(s) of the same %d-site workload on %d host threads "
                         "(oracle C port, pthreads), %.1f s" % (done, ns, nth, secs)}

    if rank == 0:
        line = {
            "metric": METRIC, "value": round(value, 4), "unit": "ns/day", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms_step, 5),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "fp32+fp64acc", "data": "synthetic (seeded fcc lattice, random orientations, %d relaxation steps of "
                    "rigid SPC/E at 1 fs with velocity rescaling to 298 K)" % args.equilibrate,
            "config": {"workload": "%s (%d sites%s), L=%.3f A, cutoff %.0f A, "
                                   "alpha %.2f/A, |n|<=%d (%d k-vectors), leap-frog+SHAKE "
                                   "dt %.0f fs%s" % (
                                       " + ".join("%d %s" % (n, {"WAT": "SPC/E waters",
                                                                 "WATD": "Drude waters",
                                                                 "NA": "Na+", "CL": "Cl-"}
                                                             .get(sp, sp))
                                                  for sp, n in zip(system.species,
                                                                   system.counts)), ns,
                                       " + %d Drude shells" % int((system.qpol != 0).sum())
                                       if system.polar else "", w["L"], w["cutoff"], w["alpha"],
                                       w["kn"], fp.nkvec, w["h"] * 1000,
                                       ", ASPC k=%d + %d SCF iteration(s)" % (w["aspc_k"],
                                                                               w["scf_iter"])
                                       if system.polar else ""),
                       "model": ("SPC/E + Drude shell water" if system.polar else
                                 "SPC/E rigid water") + ", Ewald", "global_batch": world,
                       "seq_len": ns, "parallelism": "replicas x%d" % world,
                       "l2": "flushed between timed steps (256 MB write)",
                       "autotuned": tuned or "off",
                       "pair_search": ("Verlet lists, skin %.2f A" % args.skin) if args.skin > 0
                       else "cells re-binned every step",
                       "ewald_kspace": {0: "both passes tensor cores (tcgen05 TF32x3)",
                                        1: "both passes FP32 cores",
                                        2: "pass 1 FP32 cores, pass 2 tensor cores (tcgen05 TF32x3)",
                                        3: "both passes tensor cores (tcgen05 TF32x3)"}[
                                            args.kspace_engine or 0]},
            "atom_steps_per_s": round(atom_steps, 1),
            "fp64_path": {"value": round(value64, 4), "unit": "ns/day", "steps": k64},
            "mixed_over_fp64": round(value / value64, 3),
            "force_rel_rms_vs_fp64": force_err,
            "energy_err_vs_fp64": {k: float("%.3g" % v) for k, v in energy_err.items()},
            "e2e": {"value": round(e2e, 4), "unit": "ns/day",
                    "h2d_bytes_per_step": rh.nbytes + r1h.nbytes,
                    "d2h_bytes_per_step": rh.nbytes + r1h.nbytes, "steps": ke2e},
            "gpu_launches": launches,
            "roofline": {"bound": "fp32", "kernel": name, "achieved": round(achieved, 3),
                         "peak": round(peak, 3), "unit": "TFLOP/s",
                         "frac": round(achieved / peak, 4) if peak else None,
                         "traffic": traffic,
                         "peak_source": "measured FP32 FMA loop (mg_probe_fp32_tflops); "
                                        "MEASURED_PEAKS.json has no FP32 figure",
                         "avg_launch_ms": round(kavg, 5)},
            "kernel_share": shares,
            "kernel_share_note": "per-kernel CUDA-event times of a separate pass with the k-space "
                                 "and r-space chains serialised; the timed steps run them %s" % (
                                     "one after the other" if tuned.get("kspace_serial")
                                     else "concurrently on two streams"),
            "clocks": clk,
            "cpu_baseline": cpu,
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


# ---------------------------------------------------------- batch of boxes --

BATCH_WORKLOADS = {"batch256": 256}


def run_batch(args, rank, world, local):
    """256 independent LJ + point-charge ionic-fluid boxes (N 500-4000) as one
    Batch per GPU: a step is one MD step of every box (one captured graph);
    the boxes are shared over the ranks by estimated cost (no collective).
    Widom: 1e5 insertions of the neutral LJ probe into every box, timed once
    after the MD steps (one kernel launch for all boxes)."""
    import torch
    import torch.distributed as dist
    import macsimus_gb300 as M
    from macsimus_gb300 import configs, sharding

    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    nbox = BATCH_WORKLOADS[args.workload]
    allb = configs.ionic_boxes(nbox, seed=1000)
    costs = [sharding.box_cost(b["system"].ns, (b["kn"] ** 3) * 2.1, b["cutoff"], b["L"])
             for b in allb]
    mine = sharding.partition(costs, world)[rank]
    boxes = [allb[i] for i in mine]
    nsite = sum(b["system"].ns for b in boxes)

    def barrier():
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()

    engine = 0 if args.kspace_engine is None else args.kspace_engine

    def make(precision):
        return M.Batch([dict(system=b["system"], L=b["L"], cutoff=b["cutoff"], alpha=b["alpha"],
                             kappa=b["kappa"], h=b["h"], kspace_engine=engine) for b in boxes],
                       precision=precision)

    bm = make("mixed")
    # relax the lattice starts: velocity rescaling to 298 K every 10 steps
    for i, b in enumerate(boxes):
        bm.box[i].md_set_state(b["r"], b["r1"] * 0.5)
    for _ in range(args.equilibrate // 10):
        bm.md_steps(10, measure=False)
        for i, b in enumerate(boxes):
            r, r1 = bm.box[i].md_get_state()
            m = b["system"].mass[:, None]
            T = (m * (r1 / b["h"]) ** 2).sum() / (3 * len(m) - 3)
            bm.box[i].md_set_state(r, r1 * np.sqrt(298.0 / max(T, 1e-6)))
    states = [bm.box[i].md_get_state() for i in range(len(boxes))]
    # accuracy against the FP64 path on the relaxed states
    b64 = make("fp64")
    num = den = 0.0
    ek_err, ep_err = [], []
    for i in range(len(boxes)):
        fm, em = bm.box[i].forces(states[i][0], measure=True)
        fd, ed = b64.box[i].forces(states[i][0], measure=True)
        num += ((fm - fd) ** 2).sum()
        den += (fd ** 2).sum()
        ek_err.append((em["ek"] - ed["ek"]) / abs(ed["ek"]))
        ep_err.append((em["el"] + em["lj"] - ed["el"] - ed["lj"]) / abs(ed["eself"]))
    force_err = float(np.sqrt(num / den))
    # the largest per-box energy errors
    energy_err = {"ek_rel": max(ek_err, key=abs), "epot_rel_eself": max(ep_err, key=abs)}

    def timed(batch, k, warm):
        for i in range(len(boxes)):
            batch.box[i].md_set_state(*states[i])
        batch.md_steps(warm, measure=False)
        barrier()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        ms = 0.0
        launches = 0
        for _ in range(k):
            e0.record()
            batch.md_steps(1, measure=False)
            e1.record()
            e1.synchronize()
            ms += e0.elapsed_time(e1)
            launches += batch.launches
        barrier()
        return ms, launches

    gpu_index = local
    clocks = ClockSampler(gpu_index)
    clocks.start()
    ms, launches = timed(bm, args.steps, args.warmup)
    clk = clocks.stop()
    t = torch.tensor([ms], dtype=torch.float64, device="cuda")
    if world > 1:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    ms = float(t.item())
    h = boxes[0]["h"]
    value = ns_per_day(h, args.steps, ms * 1e-3)
    k64 = max(1, min(args.steps, args.fp64_steps))
    ms64, _ = timed(b64, k64, 1)
    value64 = ns_per_day(h, k64, ms64 * 1e-3)
    # Widom: 1e5 insertions per box, one launch
    nins = 100000
    barrier()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    res = bm.widom([2], n=nins, seed=7, T=298.0)
    e1.record()
    e1.synchronize()
    wms = e0.elapsed_time(e1)
    # end to end: host states in, one step, states out, every step
    host = [(torch.from_numpy(s[0].copy()).pin_memory().numpy(),
             torch.from_numpy(s[1].copy()).pin_memory().numpy()) for s in states]
    ke = max(3, min(args.steps, 20))
    barrier()
    t0 = time.perf_counter()
    for _ in range(ke):
        for i in range(len(boxes)):
            bm.box[i].md_set_state(*host[i])
        bm.md_steps(1, measure=False)
        for i in range(len(boxes)):
            bm.box[i].md_get_state(out=(host[i][0].reshape(-1), host[i][1].reshape(-1)))
    barrier()
    e2e_s = time.perf_counter() - t0
    nbytes = sum(a.nbytes + b.nbytes for a, b in host)
    # per stage of the fused step (CUDA events between the launches), and
    # the roofline of the stage with the largest share: its algorithmic
    # work over its time (Ewald passes: 8 flops per (k-vector, charge), on
    # the tensor cores as TF32 products, three MMAs per product, at half
    # the bf16 rate; the pair terms: 45 flops per in-cutoff pair, FP32)
    for i in range(len(boxes)):
        bm.box[i].md_set_state(*states[i])
    stages = bm.profile(5) if bm.fused else {}
    fp32_peak = M.fp32_peak_tflops()
    nkq = sum(bm.box[i].nkvec * int((b["system"].q != 0).sum()) for i, b in enumerate(boxes))
    npair = sum(b["system"].ns * (b["system"].ns - 1) / 2 *
                (4.0 / 3.0 * math.pi * b["cutoff"] ** 3) / np.prod(np.broadcast_to(b["L"], 3))
                for b in boxes)
    roof = None
    if stages:
        top = max(stages, key=stages.get)
        t_top = stages[top] * 1e-3
        if top in ("ewald_sk", "ewald_kforce"):
            peaks = json.load(open(os.path.join(REPO, "MEASURED_PEAKS.json"))) \
                if os.path.exists(os.path.join(REPO, "MEASURED_PEAKS.json")) else {}
            bf16 = peaks.get("bf16_tflops", 1900.0)
            achieved = FLOP_PER_KQ * nkq / t_top / 1e12
            roof = {"bound": "tensor", "kernel": "batch " + top, "achieved": round(achieved, 3),
                    "peak": bf16, "unit": "TFLOP/s", "frac": round(achieved / bf16, 4),
                    "traffic": None, "avg_launch_ms": round(stages[top], 4),
                    "peak_source": "MEASURED_PEAKS.json bf16_tflops (burst) %s; the passes run "
                                   "TF32 products (half the bf16 rate), three MMAs each" % (
                                       "measured" if peaks else "fallback")}
        else:
            achieved = (FLOP_PER_PAIR * npair if top == "pair" else 0.0) / t_top / 1e12
            roof = {"bound": "fp32", "kernel": "batch " + top, "achieved": round(achieved, 3),
                    "peak": round(fp32_peak, 3), "unit": "TFLOP/s",
                    "frac": round(achieved / fp32_peak, 4), "traffic": None,
                    "avg_launch_ms": round(stages[top], 4),
                    "peak_source": "measured FP32 FMA loop (mg_probe_fp32_tflops)"}
    shares = {k: round(v / max(sum(stages.values()), 1e-30), 4) for k, v in stages.items()}
    if rank == 0:
        print(json.dumps({
            "metric": METRIC, "value": round(value, 4), "unit": "ns/day", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms / args.steps, 4),
            "higher_is_better": True, "scaling": "strong", "vs_baseline": None,
            "dtype": "fp32+fp64acc", "data": "synthetic (seeded lattice starts, %d steps of "
            "relaxation with velocity rescaling)" % args.equilibrate,
            "config": {"workload": "%d ionic-fluid boxes (LJ + +-1 e, N 500-4000, %d sites in "
                                   "all), per-box Ewald, leap-frog dt 2 fs; Widom 1e5 "
                                   "insertions per box" % (nbox, sum(b["system"].ns for b in allb)),
                       "boxes_on_rank0": len(boxes),
                       "ewald_kspace": {0: "tensor cores where the tiles fit", 1: "FP32 cores",
                                        2: "pass 2 on tensor cores", 3: "tensor cores"}[engine],
                       "l2": "inputs larger than L2 (per-step working set > 129 MB)"},
            "atom_steps_per_s": round(world * nsite * args.steps / (ms * 1e-3), 1),
            "fp64_path": {"value": round(value64, 4), "unit": "ns/day", "steps": k64},
            "mixed_over_fp64": round(value / value64, 3),
            "force_rel_rms_vs_fp64": force_err,
            "energy_err_vs_fp64": {k: float("%.3g" % v) for k, v in energy_err.items()},
            "widom": {"insertions_per_s": round(len(boxes) * nins / (wms * 1e-3), 1),
                      "ms": round(wms, 3), "mu_K_box0": res[0]["mu"]},
            "e2e": {"value": round(ns_per_day(h, ke, e2e_s), 4), "unit": "ns/day",
                    "h2d_bytes_per_step": nbytes, "d2h_bytes_per_step": nbytes, "steps": ke},
            "gpu_launches": launches,
            "roofline": roof,
            "kernel_share": shares,
            "kernel_share_note": "stages of the fused step (one launch per kernel over all "
                                 "boxes), CUDA events between the launches, 5 steps",
            "clocks": clk, "cpu_baseline": None,
        }), flush=True)
    bm.close()
    b64.close()
    if world > 1:
        dist.destroy_process_group()


# ---------------------------------------------------------- reference arm --

def run_reference(args, rank, world):
    """The reference's CPU algorithm on the host cores.  The reference cook
    binaries are compiled from the reference sources, which do not exist on
    the GPU host (and an x86 build cannot run there), so this arm times the
    oracle's C restatement of the same algorithm with all host threads."""
    if rank != 0:
        return
    from macsimus_gb300 import configs
    w = configs.workload(args.workload, seed=1000)
    nth = os.cpu_count() or 1
    if args.warmup > 0:
        cpu_md_steps(w, 1, 1e9, nth)
    done, secs = cpu_md_steps(w, args.steps, args.ref_budget, nth)
    v = ns_per_day(w["h"], done, secs)
    ns = w["system"].ns
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": round(v, 6), "unit": "ns/day",
        "n_gpus": world, "steps": args.steps, "steps_timed": done, "warmup": args.warmup,
        "ms_per_step": round(secs / done * 1e3, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "fp64", "data": "synthetic",
        "config": {"workload": "%s: %d molecules (%d sites), L=%.3f A" % (
            args.workload, w["system"].nmol, ns, w["L"])},
        "cpu_baseline": {"value": round(v, 6), "unit": "ns/day", "cores": nth, "kind": "port",
                         "sample": "%d MD step(s) of the full workload (time box %.0f s)"
                                   % (done, args.ref_budget)},
        "e2e": {"value": round(v, 6), "unit": "ns/day", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default=WORKLOAD)
    ap.add_argument("--fp64-steps", type=int, default=5)
    ap.add_argument("--cpu-budget", type=float, default=12.0,
                    help="seconds of CPU work in the cpu_baseline sample (whole MD steps)")
    ap.add_argument("--ref-budget", type=float, default=150.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-autotune", action="store_true")
    ap.add_argument("--kspace-engine", type=int, default=None,
                    help="Ewald engine of the FP32 path: 0 tensor cores where they fit, 1 FP32 "
                         "cores, 2 tensor-core pass 2 only, 3 tensor cores for both passes "
                         "(default 0: one launch per pass over all boxes of a batch, the "
                         "boxes whose tiles do not fit on the FP32 cores)")
    ap.add_argument("--skin", type=float, default=0.0,
                    help="> 0: Verlet lists of cutoff+skin instead of cells re-binned every step")
    ap.add_argument("--equilibrate", type=int, default=400,
                    help="relax the lattice start (rigid molecules, velocity rescaling)")
    ap.add_argument("--pair-variant", type=int, default=None,
                    help="FP32 pair kernel (mg_params.pair_variant; 8 = the group kernel, "
                         "9 and 10 its half-shell forms), "
                         "instead of the autotuner's choice")
    ap.add_argument("--cells", type=int, default=None,
                    help="cells per cutoff instead of the autotuner's choice")
    ap.add_argument("--kspace-serial", type=int, default=None, choices=[0, 1],
                    help="1: the Ewald chain after the r-space chain, 0: beside it on a second "
                         "stream, instead of the autotuner's choice")
    args = ap.parse_args()
    if args.warmup < 3 and args.impl == "ours":
        args.warmup = 3
    rank, world, local = env_rank()
    if args.impl == "reference":
        run_reference(args, rank, world)
    elif args.workload in BATCH_WORKLOADS:
        run_batch(args, rank, world, local)
    else:
        run_ours(args, rank, world, local)


if __name__ == "__main__":
    main()
