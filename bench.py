"""GNLSE ensemble benchmark: solves/s of the ragged supercontinuum ensemble on one GB300.

A step is one complete solve of the 256-member noise ensemble (2^12 / 2^13 /
2^14-point grids, 5-20 cm, 2-15 kW, 30-120 fs sech + one photon per mode,
ARK4IP at 1e-6) through the fused engine.  ``value`` is whole-job solves/s with
the inputs resident in HBM (each step restores the inputs device-to-device,
resets the per-member state and propagates every member to its fibre end);
``e2e`` is the same metric through the C ABI's host-buffer entry point
(host->device copy of the inputs and device->host copy of the outputs inside
the timed region).

The timed precision defaults to ``df`` (double-float transforms, nonlinear term and
state), the mode whose spectral error against FP64 stays below the metric's 1e-4 on
every member.  Untimed by the headline, one full-ensemble solve each in ``fp64`` and
``mixed`` (complex64 transforms) gives the FP64 reference of every member, their
solves/s and the mixed mode's per-member errors.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--precision df|mixed|fp32|fp64]
    python bench.py --impl reference ...   # the CPU reference path (FP64 oracle), all cores
"""

import argparse
import json
import math
import multiprocessing as mp
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "GNLSE ensemble solves/s on 1 GB300 (fused vs plain, <=1e-4 rel spectral err)"
UNIT = "solves/s"
DTYPE = {"fp32": "c64", "mixed": "c64+df-state", "fp64": "c128", "df": "df-c64x2"}
KERNEL_R = {"fp32": ("float", "false"), "mixed": ("float", "true"), "fp64": ("double", "false"),
            "df": ("ddf", "false")}
WORKLOAD = "sc_ensemble_256_ragged_2^12-2^14_ark4ip_1e-6"
L2_FLUSH_BYTES = 256 << 20
ENSEMBLE_SEED = 20261203  # sc_ensemble's default seed: rank 0 is the reference ensemble
# dram__bytes_read.sum + dram__bytes_write.sum per ARK4IP attempt of one member, from
# one ncu capture of the class launch on a saturated GPU (608 members x 4 attempts of the
# 2^14 grid, profiles/gnlse_kernel_df_m11_c8_saturated.md); scales the dominant
# launch's traffic by its attempts
DRAM_BYTES_PER_ATTEMPT = {("df", 11, 8): (0.715539456e9 + 3.931759e9) / 2432}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="df", choices=["df", "mixed", "fp32", "fp64"])
    ap.add_argument("--members", type=int, default=256)
    ap.add_argument("--no-legs", dest="legs", action="store_false",
                    help="skip the untimed full-ensemble fp64 and mixed solves (and with them "
                         "the per-member accuracy against FP64)")
    ap.add_argument("--e2e-steps", type=int, default=3,
                    help="steps of the end-to-end (host buffer) measurement (at most --steps)")
    ap.add_argument("--cpu-sample-s", type=float, default=12.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--plain-attempts", type=int, default=20,
                    help="attempts per grid size timed on the plain single-instance GPU path")
    ap.add_argument("--surrogate-train", type=int, default=2000,
                    help="training pulses of the surrogate leg (0: skip it)")
    ap.add_argument("--batched-iterations", type=int, default=12,
                    help="timed iterations per grid and batch size of the batched library "
                         "comparator (0: skip it)")
    ap.add_argument("--no-autotune", dest="autotune", action="store_false",
                    help="use the library's built-in class costs instead of measuring them first")
    ap.add_argument("--no-graph", dest="graph", action="store_false",
                    help="launch the timed steps eagerly instead of replaying a CUDA graph")
    ap.add_argument("--cluster", default="",
                    help="cluster size per grid size, e.g. '16384:4,8192:2' (default: the "
                         "library's choice)")
    ap.add_argument("--profile-attempts", type=int, default=0,
                    help="profiling only: run W+K launches of at most this many attempts per "
                         "member and exit (short kernels for ncu); prints no bench line")
    return ap.parse_args()


# ----------------------------------------------------------------------------
# CPU reference path (FP64 oracle restatement of pyofss ARK4IP), bounded samples
# ----------------------------------------------------------------------------
def _cpu_attempts_worker(args):
    member, n_members, attempts = args
    import numpy as np  # noqa: F401
    from oracle import gnlse_oracle as go
    from pyofsschanged_gb300.ensemble import FIBRE_835, sc_ensemble
    members, domains, fields = sc_ensemble(n_members)
    m = members[member]
    d = domains[m.n]
    grid = go.Grid(bit_width=d.bit_width, samples_per_bit=d.samples_per_bit, centre_nu=d.centre_nu)
    p = go.Propagator(grid, m.length, **FIBRE_835)
    t0 = time.perf_counter()
    _, info = p.adaptive(fields[member].copy(), 1e-6, max_attempts=attempts)
    return m.n, info["attempts"], time.perf_counter() - t0


def cpu_sample(n_members, cores, budget_s, attempts_per_member=None):
    """Time the oracle on all `cores` at once: per-attempt seconds for each grid size."""
    from pyofsschanged_gb300.ensemble import sc_ensemble
    members, _, _ = sc_ensemble(n_members)
    by_n = {}
    for i, m in enumerate(members):
        by_n.setdefault(m.n, []).append(i)
    # per-attempt cost on one core ~ 3 evals x (1.1, 2.4, 8.4) ms at 2^12, 2^13, 2^14
    est = {4096: 3 * 1.2e-3, 8192: 3 * 2.6e-3, 16384: 3 * 9.0e-3}
    jobs = []
    sizes = sorted(by_n)
    for k in range(cores):
        n = sizes[k % len(sizes)]
        mem = by_n[n][(k // len(sizes)) % len(by_n[n])]
        att = attempts_per_member or max(4, int(budget_s / est.get(n, 0.03)))
        jobs.append((mem, n_members, att))
    ctx = mp.get_context("spawn")
    t0 = time.perf_counter()
    with ctx.Pool(cores) as pool:
        res = pool.map(_cpu_attempts_worker, jobs)
    wall = time.perf_counter() - t0
    per_att = {}
    for n, att, sec in res:
        per_att.setdefault(n, []).append(sec / max(att, 1))
    per_att = {n: statistics.median(v) for n, v in per_att.items()}
    total_att = sum(a for _, a, _ in res)
    return per_att, wall, total_att, jobs


def cpu_solves_per_s(per_att, attempts_by_member, sizes_by_member, cores):
    """Whole-machine solves/s: `cores` independent solves at the sampled per-attempt cost."""
    t_solves = [attempts_by_member[i] * per_att[sizes_by_member[i]] for i in range(len(sizes_by_member))]
    mean_t = sum(t_solves) / len(t_solves)
    return cores / mean_t


def load_costs(n_members):
    path = os.path.join(ROOT, "tests", "golden", "ensemble_costs.json")
    with open(path) as f:
        c = json.load(f)
    res = c["results"]
    if len(res) < n_members:
        raise RuntimeError("ensemble_costs.json covers fewer members than requested")
    return [r["attempts"] for r in res[:n_members]], [r["n"] for r in res[:n_members]]


def spectral_power_db_error(out_t, ref_t, floor_db=-40.0):
    """Largest |10 log10(P_out / P_ref)| over the spectral bins within ``floor_db`` of the
    reference spectrum's peak (P = |fft(A)|^2 of the time-domain fields), in dB."""
    import numpy as np
    p_ref = np.abs(np.fft.ifft(ref_t)) ** 2
    p_out = np.abs(np.fft.ifft(out_t)) ** 2
    band = p_ref >= p_ref.max() * 10.0 ** (floor_db / 10.0)
    if not band.any():
        return 0.0
    with np.errstate(divide="ignore"):
        d = 10.0 * np.log10(np.maximum(p_out[band], 1e-300) / p_ref[band])
    return float(np.max(np.abs(d)))


def batched_library_leg(a, members, domains, fields, stats, value, dev):
    """Solves/s of the batched library ARK4IP (pyofsschanged_gb300.batched_library) for
    this ensemble: t(B) = t0 + B t1 per batched attempt from two timed batch sizes per
    grid, summed over the attempt counts of the members (one grid after another)."""
    import numpy as np
    import torch
    from pyofsschanged_gb300.batched_library import BatchedARK4IP
    from pyofsschanged_gb300.ensemble import FIBRE_835
    from pyofsschanged_gb300.operators import GridTables
    cdt = torch.complex64 if a.precision in ("mixed", "fp32") else torch.complex128
    total_s, ideal_s, per_grid = 0.0, 0.0, {}
    for n in sorted(domains):
        idx = [i for i, m in enumerate(members) if m.n == n]
        b = BatchedARK4IP(GridTables(domains[n], **FIBRE_835), dtype=cdt, device=dev)
        big = torch.as_tensor(np.array([fields[i] for i in idx]))
        lengths = [1.0] * len(idx)  # long fibres: no member finishes inside the sample
        t_b = {}
        for B in (len(idx), 8):
            b.propagate(big[:B], lengths[:B], 1e-6, max_iterations=2)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            b.propagate(big[:B], lengths[:B], 1e-6, max_iterations=a.batched_iterations)
            torch.cuda.synchronize()
            t_b[B] = (time.perf_counter() - t0) / a.batched_iterations
        Bf = len(idx)
        t1 = (t_b[Bf] - t_b[8]) / (Bf - 8) if Bf > 8 else t_b[Bf] / Bf
        t0c = max(0.0, t_b[8] - 8 * t1)
        att = np.array([stats[i]["attempts"] for i in idx])
        iters = int(att.max())
        active = np.array([(att > k).sum() for k in range(iters)])
        grid_s = float(np.sum(t0c + t1 * active))
        total_s += grid_s
        ideal_s += float(t1 * active.sum())
        per_grid[str(n)] = {"members": Bf, "s_per_iteration_full_batch": t_b[Bf],
                            "s_per_iteration_batch8": t_b[8], "solve_s": grid_s}
    v = len(members) / total_s
    # the same without the fixed per-iteration cost (launches, host synchronisation): the
    # batched library approach's bound if all of that overhead were hidden
    vi = len(members) / ideal_s
    return {"value": v, "unit": UNIT, "fused_over_batched": value / v,
            "value_without_fixed_overhead": vi, "fused_over_batched_without_fixed_overhead": value / vi,
            "dtype": "c128" if cdt == torch.complex128 else "c64", "per_grid": per_grid,
            "sample": f"{a.batched_iterations} batched ARK4IP attempts per grid at the full batch "
                      "and at 8 members (torch.fft/cuFFT per reference fft call, every member "
                      "of a grid in one call), t(B) = t0 + B t1 summed over this run's attempt "
                      "counts, grids one after another"}


def replay_experiment(a, members, domains, fields, leg_out, local, count=8):
    """The mixed mode's worst members re-run on the fp64 plan's own accepted step sequence
    (gnlse_set_replay): their error against fp64 with the step-size decisions taken out,
    beside the error of the mixed run with its own controller."""
    import numpy as np
    from pyofsschanged_gb300.engine import Plan
    from pyofsschanged_gb300.ensemble import ensemble_plan_inputs
    ref, mixed = leg_out["fp64"], leg_out["mixed"]

    def err(o, r):
        return float(np.linalg.norm(np.fft.ifft(o) - np.fft.ifft(r)) / np.linalg.norm(np.fft.ifft(r)))

    worst = sorted(range(len(members)), key=lambda i: -err(mixed[i], ref[i]))[:count]
    sub = [members[i] for i in worst]
    g, inst = ensemble_plan_inputs(sub, {n: domains[n] for n in set(m.n for m in sub)})
    p64 = Plan(g, inst, precision="fp64", device=local)
    for j in range(len(sub)):
        p64.set_step_log(j, 100000)
    f64 = p64.pack([fields[i] for i in worst])
    p64.propagate(f64)
    st64 = p64.stats()
    logs = [p64.step_log(j, st64) for j in range(len(sub))]
    out64 = [x.cpu().numpy() for x in p64.unpack(f64)]
    pm = Plan(g, inst, precision="mixed", device=local)
    for j in range(len(sub)):
        pm.set_replay(j, logs[j][:, 1])
    fm = pm.pack([fields[i] for i in worst])
    pm.propagate(fm)
    outm = [x.cpu().numpy().astype(complex) for x in pm.unpack(fm)]
    rows = {}
    for j, i in enumerate(worst):
        rows[str(i)] = {"n": members[i].n, "steps": int(len(logs[j])),
                        "mixed_own_controller": float("%.3e" % err(mixed[i], ref[i])),
                        "mixed_on_fp64_steps": float("%.3e" % err(outm[j], out64[j]))}
    return rows


def amplifier_leg(local):
    """The 2^16-point amplifier (pyofsschanged_gb300.amplifier): one 3 m ARK4IP solve per
    precision on its cluster class, timed with CUDA events, with the df and mixed outputs'
    spectral error against the fp64 one."""
    import numpy as np
    import torch
    from pyofsschanged_gb300.amplifier import FIBRE, LENGTH_KM, amplifier_input
    from pyofsschanged_gb300.engine import Instance, Plan
    from pyofsschanged_gb300.operators import GridTables
    d, a0 = amplifier_input()
    res, outs = {}, {}
    for prec, cl in (("df", 16), ("mixed", 8), ("fp64", 16)):
        g = GridTables(d, length=LENGTH_KM, cluster=cl, **FIBRE)
        plan = Plan([g], [Instance(0, method="ark4ip", length=LENGTH_KM, local_error=1e-6)],
                    precision=prec, device=local)
        f = plan.pack([a0])
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        plan.propagate(f)
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        st = plan.stats()[0]
        assert st["status"] == 0 and st["finished"], f"amplifier {prec}: status {st['status']}"
        outs[prec] = plan.unpack(f)[0].cpu().numpy().astype(complex)
        vsz = 16
        res[prec] = {"solve_ms": ms, "solves_per_s": 1e3 / ms, "attempts": st["attempts"],
                     "evals": st["evals"], "class": f"{g.n // cl} points x {cl} CTAs",
                     "energy_out_nJ": st["energy_out"],
                     "hbm_alg_gbs": st["evals"] * 2 * g.n * vsz / (ms * 1e-3) / 1e9}
    ref = np.fft.ifft(outs["fp64"])
    for prec in ("df", "mixed"):
        res[prec]["spectral_err_vs_fp64"] = float(
            np.linalg.norm(np.fft.ifft(outs[prec]) - ref) / np.linalg.norm(ref))
    res["workload"] = ("2^16 points, 100 ps at 1030 nm, 1 ps 100 W Gaussian with 2 ps^2 chirp, 3 m "
                       "saturable gain 39.09 dB / 5 nJ / 40 nm, Raman + self-steepening, ARK4IP 1e-6")
    return res


def run_reference(a):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    cores = os.cpu_count() or 1
    attempts, sizes = load_costs(a.members)
    values, walls = [], []
    per_step = max(2.0, a.cpu_sample_s / 2)
    for s in range(a.warmup + a.steps):
        per_att, wall, tot, jobs = cpu_sample(a.members, cores, per_step)
        if s >= a.warmup:
            values.append(cpu_solves_per_s(per_att, attempts, sizes, cores))
            walls.append(wall)
    v = statistics.median(values)
    sample = (f"per step: {cores} oracle processes (one per core) each ran a bounded number of "
              f"ARK4IP attempts (~{per_step:.0f} s) of one ensemble member; per-attempt cost per "
              f"grid size x the members' full attempt counts (tests/golden/ensemble_costs.json). "
              f"The oracle is a bit-exact restatement of the reference's ARK4IP whose per-attempt "
              f"cost is within 0.92-1.00x of the unmodified reference's on one core "
              f"(tests/golden/reference_costs.json); the reference itself cannot run here")
    line = {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": a.gpus, "steps": a.steps,
            "warmup": a.warmup, "ms_per_step": 1e3 * statistics.mean(walls),
            "ms_per_ensemble_solve_extrapolated": 1e3 * a.members / v, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "c128", "data": "synthetic",
            "config": {"workload": WORKLOAD, "members": a.members},
            "impl": "reference",
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


# ----------------------------------------------------------------------------
# GPU arm
# ----------------------------------------------------------------------------
class ClockSampler:
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.QUERY}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as f:
            for line in f:
                parts = [x.strip() for x in line.split(",")]
                if len(parts) < 9:
                    continue
                try:
                    sm.append(float(parts[1]))
                    mx.append(float(parts[2]))
                except ValueError:
                    continue
                for nm, val in zip(names, parts[5:9]):
                    if val.lower() == "active":
                        reasons.add(nm)
        os.unlink(self.path)
        if not sm:
            return None
        busy = [s for s in sm if s > 0.5 * max(sm)] or sm
        return {"sm_mhz": statistics.median(busy), "sm_max_mhz": max(mx),
                "reasons": sorted(reasons), "samples": len(sm)}


def run_ours(a):
    import numpy as np
    import torch
    import torch.distributed as dist

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)

    cpu_line = None
    from pyofsschanged_gb300.engine import Plan
    from pyofsschanged_gb300.ensemble import ensemble_plan_inputs, sc_ensemble

    # each rank propagates its own shard of a world x members ensemble (seeded per
    # rank; weak scaling, no collective during propagation)
    members, domains, fields = sc_ensemble(a.members, seed=ENSEMBLE_SEED + rank)
    cluster = {int(k): int(v) for k, v in (kv.split(":") for kv in a.cluster.split(",") if kv)}
    grids, inst = ensemble_plan_inputs(members, domains, cluster=cluster)
    tuned = None
    if a.autotune and not cluster:
        # measured SM time per attempt of every compiled class of each grid (untimed)
        from pyofsschanged_gb300.autotune import autotune
        samples = {}
        for g in grids:
            idx = [i for i, m in enumerate(members) if m.n == g.n][:8]
            samples[g.n] = (g, [fields[i] for i in idx])
        tuned = {f"{n}:{c}": round(us, 1) for (n, c), us in
                 autotune(samples, a.precision, device=local).items()}
    plan = Plan(grids, inst, precision=a.precision, device=local)
    src = plan.pack(fields)
    work = torch.empty_like(src)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream(dev)

    def barrier():
        if world > 1:
            dist.barrier()

    def step():
        work.copy_(src)
        plan.propagate(work)  # on the current stream (the capture stream under a graph)
        flush.fill_(1.0)  # write > L2 between steps

    if a.profile_attempts > 0:
        work.copy_(src)
        plan.reset(stream)
        for _ in range(a.warmup + a.steps):
            plan.propagate(work, max_attempts=a.profile_attempts, stream=stream, reset=False)
        torch.cuda.synchronize()
        print(json.dumps({"profile_attempts": a.profile_attempts, "launches": a.warmup + a.steps,
                          "classes": len(plan.class_times())}))
        return 0

    plan.set_timing(True)
    for _ in range(a.warmup):
        step()
    torch.cuda.synchronize()
    stats_w = plan.stats()
    graph = None
    if a.graph:
        # one timed step = one replay of the captured step (input copy, every class
        # launch on its forked stream with its timing events, L2 flush)
        graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(graph):
            step()
        torch.cuda.synchronize()
    clocks = ClockSampler(local)
    class_ms = []
    barrier()
    torch.cuda.synchronize()
    clocks.start()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(a.steps):
        if graph is not None:
            graph.replay()
        else:
            step()
        class_ms.append(plan.class_times())
    e1.record(stream)
    torch.cuda.synchronize()
    ck = clocks.stop()
    barrier()
    ms_total = e0.elapsed_time(e1)
    if world > 1:
        t = torch.tensor([ms_total], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms_total = float(t.item())
    stats = plan.stats()
    assert all(s["status"] == 0 and s["finished"] for s in stats), "a member did not finish"
    ms_step = ms_total / a.steps
    value = world * a.members * a.steps / (ms_total * 1e-3)

    # ensemble coherence |g12| over every rank's members (untimed): one all-reduce of the
    # spectral sums, the spectra stay on their ranks
    from pyofsschanged_gb300.ensemble import coherence_g12, coherence_g12_distributed, common_spectra
    spectra = common_spectra([x.cpu().numpy().astype(complex) for x in plan.unpack(work)])
    g12 = (coherence_g12_distributed(spectra, n_bins=spectra.shape[1]) if world > 1
           else coherence_g12(spectra))
    power = np.sum(np.abs(spectra) ** 2, axis=0)
    coherence = {"members": world * a.members,
                 "g12_power_weighted": float(np.sum(g12 * power) / np.sum(power))}

    # roofline of the dominant launch: the class launch with the most algorithmic
    # bytes (RK4IP evaluations x 2 x N x element size), timed by its own CUDA events
    vsz = 8 if a.precision == "fp32" else 16
    members_of = plan.class_members()
    launches_t = class_ms[-1]
    best = None
    for k, (logm, c, cnt, _) in enumerate(launches_t):
        ids = members_of[k]
        n = (1 << logm) * c
        b = sum(stats[i]["evals"] * 2 * n * vsz for i in ids)
        if best is None or b > best[0]:
            best = (b, k, logm, c, n, ids)
    alg_bytes, dom_k, dom_logm, dom_c, dom_n, dom_ids = best
    dom_ms = statistics.mean(st[dom_k][3] for st in class_ms)
    peaks = {}
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peaks = json.load(f)
    except OSError:
        pass
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    achieved = alg_bytes / (dom_ms * 1e-3) / 1e9
    fft_flops = sum(stats[i]["evals"] * 16 * 5.0 * dom_n * math.log2(dom_n) for i in dom_ids)
    # DRAM bytes per attempt from one ncu capture of this class, scaled to this launch
    per_attempt = DRAM_BYTES_PER_ATTEMPT.get((a.precision, dom_logm, dom_c))
    traffic = per_attempt * sum(stats[i]["attempts"] for i in dom_ids) if per_attempt else None
    roofline = {"bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                "frac": achieved / hbm_peak, "traffic": traffic,
                "kernel": f"gnlse_kernel<{KERNEL_R[a.precision][0]},{dom_logm},{dom_c},{KERNEL_R[a.precision][1]}>",
                "launch_ms": dom_ms, "alg_bytes_per_launch": alg_bytes, "members": len(dom_ids),
                "peak_source": "MEASURED_PEAKS.json" if peaks else "fallback",
                "fft_gflops": fft_flops / (dom_ms * 1e-3) / 1e9}

    # end to end through the C ABI host-buffer entry point
    npdt = np.complex64 if a.precision == "fp32" else np.complex128
    host_in = src.cpu().numpy().astype(npdt)
    host_out = np.empty_like(host_in)
    plan.propagate_host(host_in, host_out)
    e2e_steps = max(1, min(a.steps, a.e2e_steps))
    barrier()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        plan.propagate_host(host_in, host_out)
    e2e_s = time.perf_counter() - t0
    if world > 1:
        t = torch.tensor([e2e_s], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_s = float(t.item())
    e2e = {"value": world * a.members * e2e_steps / e2e_s, "unit": UNIT,
           "h2d_bytes_per_step": int(host_in.nbytes), "d2h_bytes_per_step": int(host_out.nbytes),
           "steps": e2e_steps}

    # Untimed by the headline: one full-ensemble solve in fp64 (the accuracy reference of
    # every member, and the FP64 solves/s) and one in mixed precision, each on its own
    # autotuned plan, timed with CUDA events around the propagate call.
    acc, legs = None, {}
    if a.legs and rank == 0:
        out = [x.cpu().numpy().astype(complex) for x in plan.unpack(work)]
        leg_out = {a.precision: out}
        for prec in ("fp64", "mixed"):
            if prec == a.precision:
                legs[prec] = {"value": value, "unit": UNIT, "timed": "headline"}
                continue
            if a.autotune and not cluster:
                from pyofsschanged_gb300.autotune import autotune
                samples = {g.n: (g, [fields[i] for i, m in enumerate(members) if m.n == g.n][:8])
                           for g in grids}
                autotune(samples, prec, device=local)
            lp = Plan(grids, inst, precision=prec, device=local)
            lf = lp.pack(fields)
            torch.cuda.synchronize()
            l0, l1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            l0.record(stream)
            lp.propagate(lf)
            l1.record(stream)
            torch.cuda.synchronize()
            lms = l0.elapsed_time(l1)
            lst = lp.stats()
            assert all(x["status"] == 0 and x["finished"] for x in lst), f"{prec}: a member did not finish"
            leg_out[prec] = [x.cpu().numpy().astype(complex) for x in lp.unpack(lf)]
            legs[prec] = {"value": a.members / (lms * 1e-3), "unit": UNIT, "ms": lms,
                          "attempts": int(sum(x["attempts"] for x in lst)), "steps": 1,
                          "dtype": DTYPE[prec]}
            del lp, lf
        ref = leg_out["fp64"]
        sizes = [m.n for m in members]

        def accuracy(outs):
            errs = [float(np.linalg.norm(np.fft.ifft(o) - np.fft.ifft(r)) / np.linalg.norm(np.fft.ifft(r)))
                    for o, r in zip(outs, ref)]
            db = [spectral_power_db_error(o, r) for o, r in zip(outs, ref)]
            worst = sorted(range(len(errs)), key=lambda i: -errs[i])[:8]
            by_grid = {str(n): max(e for e, m in zip(errs, sizes) if m == n) for n in sorted(set(sizes))}
            return {"members": len(errs), "median": statistics.median(errs), "max": max(errs),
                    "frac_le_1e-4": sum(e <= 1e-4 for e in errs) / len(errs),
                    "n_above_1e-4": sum(e > 1e-4 for e in errs), "max_by_grid": by_grid,
                    "worst_members": {str(i): float("%.3e" % errs[i]) for i in worst},
                    "spectral_power_db_max_within_40db": max(db)}

        if a.precision != "fp64":
            acc = accuracy(out)
            acc["vs"] = "fp64 engine plan on the same inputs, every member"
        if "mixed" in leg_out and a.precision != "mixed":
            legs["mixed"]["accuracy_vs_fp64"] = accuracy(leg_out["mixed"])
            legs["mixed"]["replay_of_fp64_steps"] = replay_experiment(
                a, members, domains, fields, leg_out, local)
        legs["fp64"]["accuracy"] = ("the reference precision (tests/test_gpu_parity.py and "
                                    "tests/test_gpu_ensemble_parity.py: <= 1e-9 against the FP64 oracle)")

    # plain single-instance GPU path (one library call per reference operation),
    # bounded per-attempt samples per grid size x this run's per-member attempt counts
    plain = None
    if rank == 0 and a.plain_attempts > 0:
        from pyofsschanged_gb300.ensemble import FIBRE_835
        from pyofsschanged_gb300.operators import GridTables
        from pyofsschanged_gb300.plain import PlainRK4IP
        per_att = {}
        for n in sorted(domains):
            i = next(k for k, m in enumerate(members) if m.n == n)
            pp = PlainRK4IP(GridTables(domains[n], **FIBRE_835), members[i].length)
            a0 = torch.as_tensor(fields[i]).to(dev)
            pp.adaptive(a0, 1e-6, max_attempts=2)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            _, att, _ = pp.adaptive(a0, 1e-6, max_attempts=a.plain_attempts)
            torch.cuda.synchronize()
            per_att[n] = (time.perf_counter() - t0) / att
        t_solve = [s["attempts"] * per_att[plan.grids[plan.instances[i].grid].n]
                   for i, s in enumerate(stats)]
        pv = 1.0 / (sum(t_solve) / len(t_solve))
        plain = {"value": pv, "unit": UNIT, "fused_over_plain": value / pv,
                 "sample": f"{a.plain_attempts} ARK4IP attempts per grid size, complex128, "
                           "torch.fft/cuFFT per reference fft call, host read-back per attempt",
                 "s_per_attempt": {str(k): v for k, v in per_att.items()}}

    # batched library comparator: the same ARK4IP on torch.fft (cuFFT) over all members of
    # a grid at once, per-member h as elementwise arrays, finished members leaving the batch;
    # per-iteration cost t(B) = t0 + B t1 measured at two batch sizes per grid, summed over
    # the iterations the members' attempt counts (this run's) need, grids one after another
    amp = amplifier_leg(local) if (a.legs and rank == 0) else None

    # learned surrogate with RK4IP fallback, on a reduced training set (the full 20k-sample
    # experiment is python -m pyofsschanged_gb300.surrogate_run): acceptance and solves/s
    # against the engine on the same held-out pulses
    sur = None
    if a.legs and rank == 0 and a.surrogate_train > 0:
        from pyofsschanged_gb300 import surrogate_run
        r = surrogate_run.run(["--train", str(a.surrogate_train), "--calib", "200", "--test", "500",
                               "--epochs", "3"])
        sur = {"train": a.surrogate_train, "test": 500, "epochs": 3, "train_s": r["train_s"],
               "test_error": r["test_error"], "engine_solves_per_s": r["engine_solves_per_s_test"],
               "with_fallback": r["surrogate_with_fallback"]}

    batched = None
    if rank == 0 and a.batched_iterations > 0:
        batched = batched_library_leg(a, members, domains, fields, stats, value, dev)

    if rank == 0 and not a.no_cpu:
        per_att, wall, tot, jobs = cpu_sample(a.members, os.cpu_count() or 1, a.cpu_sample_s)
        attempts = [s["attempts"] for s in stats]
        sizes = [plan.grids[plan.instances[i].grid].n for i in range(len(stats))]
        cores = os.cpu_count() or 1
        v = cpu_solves_per_s(per_att, attempts, sizes, cores)
        cpu_line = {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                    "sample": (f"{cores} concurrent oracle (FP64 numpy restatement of pyofss "
                               f"ARK4IP) processes, {tot} attempts in {wall:.1f} s; per-attempt "
                               f"cost per grid size x this run's per-member attempt counts")}
    launches = a.steps * len(class_ms[0])
    evals = sum(s["evals"] for s in stats)
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": a.steps,
            "warmup": a.warmup, "ms_per_step": ms_step, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None,
            "dtype": DTYPE[a.precision], "data": "synthetic",
            "config": {"workload": WORKLOAD, "members": a.members, "precision": a.precision,
                       "grids": "2^12/2^13/2^14 mixed, dt=12.5ps/8192, 835 nm",
                       "l2": "256 MiB buffer written between steps",
                       "launch": "CUDA graph replay per step" if graph is not None else "eager",
                       "class_sm_us_per_attempt": tuned,
                       "evals_per_step": evals},
            "roofline": roofline, "cpu_baseline": cpu_line, "e2e": e2e, "clocks": ck,
            "gpu_launches": launches, "accuracy_vs_fp64": acc, "legs": legs, "plain": plain,
            "batched_library": batched, "amplifier_2e16": amp, "surrogate": sur,
            "coherence": coherence,
            "class_ms": {f"m2^{lm}_c{c}_n{cnt}": statistics.mean(st[k][3] for st in class_ms)
                         for k, (lm, c, cnt, _) in enumerate(class_ms[0])}}
    if rank == 0:
        print(json.dumps(line))
    if world > 1:
        dist.destroy_process_group()
    return 0


def main():
    a = parse()
    if a.impl == "reference":
        return run_reference(a)
    return run_ours(a)


if __name__ == "__main__":
    sys.exit(main())
