"""oxDNA2 MD throughput on one GB300: particle-steps/s of the GPU hot path.

Headline workload (default, --workload large250k): 250 single strands of 1,000 random-sequence
nucleotides (250,000 nt), grown as seeded self-avoiding random walks in a cube of side 232.08
(0.02 nt/unit^3), relaxed for 1,000 + 200 steps with the backbone force capped, then T = 300 K,
0.5 M salt, dt = 0.003, Brownian ("john") thermostat every 103 steps (diff_coeff 2.5), Verlet
skin 0.05, FP32 forces with FP64 integration.  Sub-objects report the 40,000-nucleotide plain
system (`plain40k`: 1,000 random 20-bp duplexes at 0.01 nt/unit^3, Bussi tau = 1000 applied
every step) and the 256-system parallel-tempering batch (`batched`).  Inputs are generated from a
seed (no dataset is involved).

One bench "step" is one timed iteration of M MD steps (default 200) on state resident in HBM;
L2 is flushed (a 256 MiB write) before every timed iteration, outside the timed interval.
`value` = nucleotides x MD steps / device time of the K timed iterations.  `e2e` is the same
metric through the C ABI with host buffers: every iteration uploads the state from host memory,
runs M steps and downloads the state.  The roofline is that of the force kernels (FP32
CUDA-core bound): algorithmic FLOPs per launch (every bond and every unordered pair once, the
kernels' own pair physics counted with a counting scalar type) / their CUDA-event time, against
an FP32 FMA throughput measured on the same GPU.  `batched` (rank 0, one GPU): the 256 systems
in one engine against the same systems run one at a time through the plain path.

CPU baseline and --impl reference: the reference's own Release CPU program (built from its
sources by oracle/ref/Makefile when they are present: OXDNA_REFERENCE, or the untracked copy in
baseline/_ref/oxDNA), one single-threaded process per host core on the same generated system;
where the sources are absent, the FP64 oracle restatement (oracle/) on all host threads.
--impl reference-cuda times the reference's CUDA mixed backend built from the same sources for
sm_103a, on the same system.

Multi-GPU (torchrun): the plain path does not shard; every rank runs an independent replica
(weak scaling) and rank 0 reports the summed throughput over the slowest rank's time.
"""

from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

WORKLOADS = {
    "plain40k": dict(cfg=1, scale=1.0, thermostat="bussi", newtonian_steps=1, bussi_tau=1000.0, dt=0.003,
                     desc="1000 x 20-bp duplexes (40,000 nt), cube 158.74, Bussi tau 1000"),
    "large250k": dict(cfg=2, scale=1.0, thermostat="john", newtonian_steps=103, diff_coeff=2.5, dt=0.003,
                      relax_steps=1000,
                      desc="250 x 1000-nt random-walk strands (250,000 nt), cube 232.08, Brownian n=103, "
                           "after 1000 + 200 force-capped relaxation steps"),
    "duplex24": dict(cfg=0, scale=1.0, thermostat="no", newtonian_steps=1, dt=0.005,
                     desc="one 12-bp duplex (24 nt), cube 20, NVE"),
}


# dram__bytes_read.sum + dram__bytes_write.sum of k_bonded_pairs + k_nonbonded_split per force
# launch (the MD step's variant, autotuned shape 4), from the one-kernel ncu --set full captures
# summarised in profiles/k_*_{plain40k,large250k}.md (cold caches)
FORCE_TRAFFIC = {"plain40k": 8.596992e6 + 22.528e3 + 21.910528e6 + 0.0,
                 "large250k": 34.994688e6 + 162.56e3 + 50.4192e6 + 416.512e3}


def env_rank():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("LOCAL_RANK", "0"))


def make_system(wl, seed):
    from oxdna_gb300 import generate as G
    cache = os.path.join(tempfile.gettempdir(), f"oxgb_{wl['cfg']}_{wl['scale']}_{seed}.npz")
    if os.path.exists(cache):
        d = np.load(cache)
        from oxdna_gb300 import io as oxio
        top = oxio.Topology(d["n3"], d["n5"], d["btype"], d["type"], d["strand"], int(d["nstr"]))
        return G.System(float(d["box"]), d["pos"], d["a1"], d["a3"], d["vel"], d["L"], top, float(d["T"]))
    s = G.system_for_config(wl["cfg"], seed=seed, scale=wl["scale"])
    np.savez(cache, box=s.box, pos=s.pos, a1=s.a1, a3=s.a3, vel=s.vel, L=s.L, n3=s.top.n3, n5=s.top.n5,
             btype=s.top.btype, type=s.top.type, strand=s.top.strand, nstr=s.top.n_strands, T=s.T)
    return s


def relaxed_cache_path(wl, seed):
    return os.path.join(tempfile.gettempdir(), f"oxgb_{wl['cfg']}_{wl['scale']}_{seed}_relaxed{wl.get('relax_steps', 0)}.npz")


def relax(s, wl, seed):
    """Force-capped relaxation of a generated state before it is timed: relax_steps steps with
    the backbone force capped at 5 (max_backbone_force = 5, as in the reference's relaxation
    examples), then 200 steps capped at 50, under which the bonds that thermal excursions past the
    soft cap left outside the FENE range return into it; a Brownian thermostat refreshes 10 %
    of the momenta every step and removes the heat of relaxation.  The relaxed state is cached
    beside the generated one."""
    from oxdna_gb300 import generate as G
    from oxdna_gb300 import io as oxio
    import oxdna_gb300 as ox
    n = wl.get("relax_steps", 0)
    if n <= 0:
        return s
    cache = relaxed_cache_path(wl, seed)
    if os.path.exists(cache):
        d = np.load(cache)
        return G.System(s.box, d["pos"], d["a1"], d["a3"], d["vel"], d["L"], s.top, s.T)
    pos, quat, vel, L = s.pos, s.quats(), s.vel, s.L
    for fmax, steps in ((5.0, n), (50.0, 200)):
        m = ox.MDSystem(s.box, s.top, ox.dna2_settings(s.T, 0.5, mbf_fmax=fmax),
                        ox.md_settings(dt=wl["dt"], thermostat="john", newtonian_steps=1, pt=0.1, seed=seed,
                                       precision="mixed"))
        m.set_state(pos, quat, vel, L)
        m.run(steps)
        st = m.get_state()
        m.close()
        pos, quat, vel, L = st["pos"], st["quat"], st["vel"], st["Lmom"]
    a1, _, a3 = oxio.quat_to_frame(quat)
    out = G.System(s.box, pos, a1, a3, vel, L, s.top, s.T)
    np.savez(cache, pos=out.pos, a1=out.a1, a3=out.a3, vel=out.vel, L=out.L)
    return out


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms during the timed region."""

    def __init__(self, gpu_index=0):
        self.gpu = gpu_index
        self.proc = None
        self.path = os.path.join(tempfile.gettempdir(), f"oxgb_clocks_{os.getpid()}.csv")

    def start(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                          "-lms", "200"], stdout=self.fh, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.fh.close()
        rows = [ln.split(",") for ln in open(self.path).read().strip().split("\n") if ln.strip()]
        sm = [float(r[1]) for r in rows if len(r) > 2 and r[1].strip().replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if len(r) > 2 and r[2].strip().replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            for k, nm in enumerate(names):
                if len(r) > 5 + k and r[5 + k].strip().lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(rows)}


def oracle_baseline(sysm_data, wl, nsteps, nthreads):
    """CPU FP64 oracle: nsteps full MD steps (pair search, forces, integration)."""
    sys.path.insert(0, os.path.join(HERE, "oracle"))
    import oracle
    from oxdna_gb300 import io as oxio
    s = sysm_data
    p = oracle.make_params(oracle.make_settings(s.T, 0.5))
    a1, a2, a3 = s.frames()
    N = s.N
    st = dict(pos=s.pos.copy(), quat=oxio.frame_to_quat(a1, a2, a3), vel=s.vel.copy(), Lmom=s.L.copy(),
              F=np.zeros((N, 3)), T=np.zeros((N, 3)))
    rc, F, T, Es, Ep = oracle.forces(p, s.pos, a1, a2, a3, s.top.n3, s.top.n5, s.top.type, s.top.btype, s.box,
                                     nthreads=nthreads)
    st["F"][:], st["T"][:] = F, T
    md = oracle.MD()
    md.dt = wl["dt"]
    md.thermostat = {"no": 0, "john": 1, "bussi": 2}[wl["thermostat"]]
    md.newtonian_steps = wl["newtonian_steps"]
    md.bussi_tau = wl.get("bussi_tau", 1000.0)
    md.bussi_K_t = 0.5 * 3 * (N - 1) * s.T
    md.bussi_K_r = 0.5 * 3 * N * s.T
    md.seed = 1
    md.pt = 0.01228
    md.pr = 0.0041
    t0 = time.perf_counter()
    oracle.md_run(p, md, st, s.top.n3, s.top.n5, s.top.type, s.top.btype, s.box, 0, nsteps, nthreads=nthreads)
    dt = time.perf_counter() - t0
    return N * nsteps / dt, dt


def batched_workload(seed):
    """The 256-system parallel-tempering workload (cached like make_system)."""
    from oxdna_gb300 import generate as G
    cache = os.path.join(tempfile.gettempdir(), f"oxgb_batched256_{seed}.npz")
    from oxdna_gb300 import io as oxio
    if os.path.exists(cache):
        d = np.load(cache, allow_pickle=True)
        return list(d["systems"])
    systems = G.batched_systems(256, seed=seed)
    try:
        np.savez(cache, systems=np.array(systems, dtype=object))
    except Exception:
        pass
    return systems


def batched_reference_cpu(systems, steps):
    """the reference's Release CPU program on the 256 systems, one process per host core at a
    time (the reference's own way to run many small systems), each system `steps` MD steps with
    its own temperature and the workload's Bussi thermostat; None where the reference sources are
    absent"""
    sys.path.insert(0, os.path.join(HERE, "oracle"))
    import refrun
    if refrun.reference_checkout() is None and not os.path.exists(refrun.PROGRAMS["cpu"]):
        return None
    try:
        exe = refrun.build("cpu")
        n = cpu_cores()
        r = refrun.cpu_batch_rate(exe, systems, n, steps, backend="CPU", dt=0.003, thermostat="bussi",
                                  newtonian_steps=1, bussi_tau=1000.0)
    except Exception as e:  # noqa: BLE001
        print(f"reference CPU batch baseline unavailable: {e}", file=sys.stderr)
        return None
    return {"value": r["value"], "unit": "particle-steps/s", "cores": n, "kind": "reference",
            "sample": f"the reference Release CPU program on each of the {len(systems)} systems, {n} processes at a "
                      f"time, {steps} MD steps each timed by its own step-loop timer; throughput = sum N_i / "
                      f"(sum of seconds per step / {n}) ({r['wall_s']:.0f} s wall)"}


def bench_batched(args, torch, ox, _abi, compare=True):
    """256 independent systems (16-4000 nt, duplexes and hairpins, each in its own cube at
    0.005 nt/unit^3, temperatures on a geometric 280-360 K ladder, 0.5 M, dt 0.003, Bussi tau
    1000) in one engine, with parallel-tempering swaps every 1000 steps on FP64 energies, against
    the same systems run one at a time through the plain path.  Wall-clock (host-synchronised)
    time, since the swaps involve the host."""
    from oxdna_gb300 import io as oxio
    systems = batched_workload(args.seed)
    n_tot = sum(s.N for s in systems)
    md = dict(dt=0.003, thermostat="bussi", newtonian_steps=1, bussi_tau=1000.0, seed=7, precision="mixed",
              steps_per_graph=25, autotune=not args.no_autotune, list_rebuild_node=args.list_node)

    def state(s):
        a1, a2, a3 = s.frames()
        return s.pos, oxio.frame_to_quat(a1, a2, a3), s.vel, s.L

    b = ox.MDSystem([s.box for s in systems], [s.top for s in systems], [ox.dna2_settings(s.T, 0.5) for s in systems],
                    ox.md_settings(**md))
    b.set_state(*[np.concatenate(x) for x in zip(*[state(s) for s in systems])])
    shape = b.force_shape()
    M = args.md_steps
    for _ in range(args.warmup):
        b.run(M, sync=False)
    torch.cuda.synchronize()
    temps = np.array([s.T for s in systems])
    rng = np.random.default_rng(args.seed)
    done, tried, accepted, parity = 0, 0, 0, 0
    t0 = time.perf_counter()
    for _ in range(args.steps):
        b.run(M, sync=False)
        done += M
        if done % 1000 == 0:
            temps, acc = b.replica_exchange(temps, rng, parity)
            tried += len(systems) // 2
            accepted += acc
            parity ^= 1
    torch.cuda.synchronize()
    t_batch = time.perf_counter() - t0
    _abi.check(_abi.lib().oxgb_md_status(b.handle))
    b.close()
    v_batch = n_tot * M * args.steps / t_batch
    if not compare:
        return {"value": v_batch, "unit": "particle-steps/s", "n_systems": len(systems), "n_nucleotides": n_tot,
                "md_steps": M * args.steps, "force_shape": shape}

    # the same systems through the plain path, one engine each, one after the other
    t_plain = 0.0
    for k, s in enumerate(systems):
        m = ox.MDSystem(s.box, s.top, ox.dna2_settings(s.T, 0.5), ox.md_settings(**dict(md, seed=7 + k)))
        m.set_state(*state(s))
        m.run(M)  # warm-up and graph capture
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        m.run(M)
        torch.cuda.synchronize()
        t_plain += time.perf_counter() - t1
        m.close()
    v_plain = n_tot * M / t_plain
    out_cpu = None
    if not args.no_cpu_baseline:
        out_cpu = batched_reference_cpu(systems, args.cpu_steps)
    return {"value": v_batch, "unit": "particle-steps/s", "n_systems": len(systems), "n_nucleotides": n_tot,
            "md_steps": M * args.steps, "pt_swaps_tried": tried, "pt_swaps_accepted": accepted,
            "plain_one_at_a_time": v_plain, "speedup_vs_plain": v_batch / v_plain, "force_shape": shape,
            "cpu_baseline": out_cpu,
            "description": "256 systems, 16-4000 nt log-uniform, duplexes/hairpins, 0.005 nt/unit^3, "
                           "280-360 K geometric ladder, Bussi tau 1000, PT swaps every 1000 steps; "
                           "wall clock including the swaps"}


def bench_batched_sharded(args, torch, ox, _abi, rank, world):
    """The 256-system workload split over the ranks (oxdna_gb300.pt.partition: size-balanced),
    one engine per GPU, parallel-tempering swaps every 1000 steps across all ranks (the FP64
    energies all-reduced, every rank taking the same decisions, each applying those of its own
    systems).  Total work is fixed (strong scaling); value = all nucleotides x MD steps / the
    slowest rank's wall time."""
    from oxdna_gb300 import io as oxio
    from oxdna_gb300 import pt
    systems = batched_workload(args.seed)
    mine = pt.partition([s.N for s in systems], world)[rank]
    local = [systems[k] for k in mine]
    n_tot = sum(s.N for s in systems)

    def state(s):
        a1, a2, a3 = s.frames()
        return s.pos, oxio.frame_to_quat(a1, a2, a3), s.vel, s.L

    b = ox.MDSystem([s.box for s in local], [s.top for s in local], [ox.dna2_settings(s.T, 0.5) for s in local],
                    ox.md_settings(dt=0.003, thermostat="bussi", newtonian_steps=1, bussi_tau=1000.0, seed=7 + 1000 * rank,
                                   precision="mixed", steps_per_graph=25, autotune=not args.no_autotune))
    b.set_state(*[np.concatenate(x) for x in zip(*[state(s) for s in local])])
    lad = pt.RankLadder(mine, [s.T for s in systems], seed=args.seed, device="cuda")
    M = args.md_steps
    for _ in range(args.warmup):
        b.run(M, sync=False)
    torch.cuda.synchronize()
    torch.distributed.barrier()
    t0 = time.perf_counter()
    done = 0
    for _ in range(args.steps):
        b.run(M, sync=False)
        done += M
        if done % 1000 == 0:
            lad.exchange(b)
    torch.cuda.synchronize()
    t = torch.tensor([time.perf_counter() - t0], device="cuda", dtype=torch.float64)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    _abi.check(_abi.lib().oxgb_md_status(b.handle))
    b.close()
    return {"value": n_tot * M * args.steps / float(t.item()), "unit": "particle-steps/s", "n_systems": len(systems),
            "n_nucleotides": n_tot, "md_steps": M * args.steps, "ranks": world, "scaling": "strong",
            "systems_per_rank_max": int(max(len(p) for p in pt.partition([s.N for s in systems], world))),
            "pt_swaps_tried": lad.tried, "pt_swaps_accepted": lad.accepted,
            "description": "256 systems split over the ranks (size-balanced), PT swaps across ranks every 1000 "
                           "steps; wall clock of the slowest rank"}


def cpu_cores():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def reference_cpu_baseline(s, wl, seed, steps=3, processes=None):
    """The reference's own Release CPU program (oracle/ref/Makefile, built from its sources when
    they are present) on system s: one single-threaded process per host core, each a copy of the
    same system, timed by its own step-loop timer (set-up excluded).  Returns the line's
    cpu_baseline object, or None when the reference sources are absent or the build fails (the
    FP64 oracle port then stands in)."""
    sys.path.insert(0, os.path.join(HERE, "oracle"))
    import refrun
    if refrun.reference_checkout() is None and not os.path.exists(refrun.PROGRAMS["cpu"]):
        return None
    try:
        exe = refrun.build("cpu")
    except Exception as e:  # noqa: BLE001
        print(f"reference CPU build unavailable: {e}", file=sys.stderr)
        return None
    n = processes or cpu_cores()
    thermo = dict(thermostat=wl["thermostat"], newtonian_steps=wl["newtonian_steps"],
                  diff_coeff=wl.get("diff_coeff", 2.5), bussi_tau=wl.get("bussi_tau", 1000.0))
    r = refrun.cpu_rates(exe, s, n, steps, backend="CPU", dt=wl["dt"], **thermo)
    return {"value": r["value"], "unit": "particle-steps/s", "cores": n, "kind": "reference",
            "s_per_step_per_copy": r["s_per_step"],
            "sample": f"{n} copies of the reference Release CPU program (-O3 -ffast-math, interaction DNA2) on "
                      f"the {s.N}-nt system as generated, run at the same time, one per core, {steps} MD steps "
                      f"each, timed by the program's own step-loop timer ({r['s_per_step']:.3f} s per step on "
                      f"average, {r['wall_s']:.0f} s wall with set-up)"}


def port_cpu_baseline(s, wl, nsteps):
    cores = cpu_cores()
    v, dt = oracle_baseline(s, wl, max(1, nsteps), cores)
    return {"value": v, "unit": "particle-steps/s", "cores": cores, "kind": "port",
            "sample": f"{nsteps} full MD steps of the {s.N}-nt system (FP64 oracle restatement, {cores} threads, "
                      f"{dt:.1f} s)"}


def run_reference_arm(args, wl):
    rank, world, _ = env_rank()
    if rank != 0:
        return
    s = make_system(wl, args.seed)
    per = []
    cpu = None
    for _ in range(args.steps):
        cpu = reference_cpu_baseline(s, wl, args.seed, steps=args.cpu_steps)
        if cpu is None:
            break
        per.append(cpu["value"])
        if len(per) >= max(1, args.reference_repeats):
            break
    if cpu is None:
        per = []
        for _ in range(max(1, min(args.steps, args.reference_repeats))):
            cpu = port_cpu_baseline(s, wl, args.cpu_sample_steps)
            per.append(cpu["value"])
    value = float(np.mean(per))
    cpu["value"] = value
    ms = 1e3 * cpu["s_per_step_per_copy"] if "s_per_step_per_copy" in cpu else 1e3 * s.N / value
    line = {"metric": "oxDNA2 MD particle-steps/s", "value": value, "unit": "particle-steps/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "impl": "reference",
            "config": {"workload": args.workload, "n_nucleotides": s.N, "description": WORKLOADS[args.workload]["desc"]},
            "cpu_baseline": cpu,
            "e2e": {"value": value, "unit": "particle-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "note": "ms_per_step: one MD step of one copy (copies run at the same time, one per core); "
                    "samples: " + ", ".join(f"{v:.4g}" for v in per)}
    print(json.dumps(line), flush=True)


def run_reference_cuda_arm(args, wl):
    """The reference CUDA mixed backend (backend = CUDA, backend_precision = mixed, CUDA_list =
    verlet), built from the reference's own sources for sm_103a, on the same system as our arm
    (the relaxed state when our arm has left it in the cache), timed as the wall-time difference
    of two runs; with its device-side energy of the starting configuration next to ours under
    both average-sequence well-depth conventions."""
    rank, world, _ = env_rank()
    if rank != 0:
        return
    sys.path.insert(0, os.path.join(HERE, "oracle"))
    import refrun
    try:
        exe = refrun.build("cuda")
    except Exception as e:  # noqa: BLE001
        print(json.dumps({"impl": "reference-cuda", "unavailable": str(e).splitlines()[0]}), flush=True)
        return
    s = make_system(wl, args.seed)
    cache = relaxed_cache_path(wl, args.seed)
    relaxed = os.path.exists(cache)
    if relaxed:
        from oxdna_gb300 import generate as G
        d = np.load(cache)
        s = G.System(s.box, d["pos"], d["a1"], d["a3"], d["vel"], d["L"], s.top, s.T)
    thermo = dict(thermostat=wl["thermostat"], newtonian_steps=wl["newtonian_steps"],
                  diff_coeff=wl.get("diff_coeff", 2.5), bussi_tau=wl.get("bussi_tau", 1000.0))
    a, b = args.ref_cuda_steps if args.ref_cuda_steps else (1000, 1000 + max(5000, int(2e9 / s.N)))
    r = refrun.time_steps(exe, s, a, b, backend="CUDA", dt=wl["dt"], **thermo)
    value = s.N / r["s_per_step"]
    line = {"metric": "oxDNA2 MD particle-steps/s", "value": value, "unit": "particle-steps/s", "n_gpus": 1,
            "impl": "reference-cuda", "ms_per_step": r["s_per_step"] * 1e3, "higher_is_better": True,
            "dtype": "f32", "data": "synthetic",
            "config": {"workload": args.workload, "n_nucleotides": s.N, "description": wl["desc"],
                       "state": "relaxed (as timed by our arm)" if relaxed else "as generated",
                       "backend": "CUDA, backend_precision = mixed, CUDA_list = verlet, CUDA_sort_every = 0"},
            "timing": {"steps": r["steps"], "wall_s": r["wall_s"], "own_ms_per_step": r["own_ms_per_step"]}}
    if args.ref_cuda_energy:
        try:
            line["energy_per_nucleotide"] = reference_cuda_energy_check(refrun, exe, s, wl)
        except Exception as e:  # noqa: BLE001
            line["energy_per_nucleotide"] = {"error": str(e)[-1500:]}
    print(json.dumps(line), flush=True)


def reference_cuda_energy_check(refrun, exe, s, wl):
    """the reference CUDA backend's device energy of s against ours, under the oxDNA2 and the
    reference-CUDA average-sequence well depths"""
    import torch
    torch.cuda.set_device(0)
    import oxdna_gb300 as ox
    from oxdna_gb300 import io as oxio
    e_ref = refrun.cuda_energy_per_nucleotide(exe, s)
    a1, a2, a3 = s.frames()
    q = oxio.frame_to_quat(a1, a2, a3)
    ours = {}
    for name, flag in (("oxdna2_eps", False), ("reference_cuda_eps", True)):
        m = ox.MDSystem(s.box, s.top, ox.dna2_settings(s.T, 0.5, reference_cuda_eps=flag),
                        ox.md_settings(dt=wl["dt"], precision="mixed"))
        m.set_state(s.pos, q, s.vel, s.L)
        _, _, E, _ = m.compute_forces()
        m.close()
        ours[name] = float(np.sum(E) / (2 * s.N))
    return {"reference_cuda": e_ref, "ours_oxdna2_eps": ours["oxdna2_eps"],
            "ours_reference_cuda_eps": ours["reference_cuda_eps"],
            "note": "reference CUDA_print_energy (printed to 6 decimals) vs our engine on the same configuration"}


def precision_study(args):
    """The precision study on the 40,000-nucleotide system: force, torque and per-term energy
    errors of the mixed-precision kernels against the same kernels in FP64 over `snapshots`
    snapshots taken every `every` steps of the Bussi run (and against the FP64 CPU oracle on a
    few of them), and the NVE energy drift per 10^6 steps of mixed (FP32 forces, FP64
    integration), float (FP32 forces, FP32 integration: backend_precision = float) and double
    precision."""
    import torch
    torch.cuda.set_device(0)
    import oxdna_gb300 as ox
    from oxdna_gb300 import io as oxio
    wl = WORKLOADS["plain40k"]
    s = make_system(wl, args.seed)
    a1, a2, a3 = s.frames()
    quat = oxio.frame_to_quat(a1, a2, a3)
    dna = ox.dna2_settings(s.T, 0.5)

    def engine(precision, thermostat):
        m = ox.MDSystem(s.box, s.top, dna, ox.md_settings(dt=wl["dt"], thermostat=thermostat, newtonian_steps=1,
                                                            bussi_tau=wl["bussi_tau"], seed=args.seed, precision=precision,
                                                            steps_per_graph=25))
        m.set_state(s.pos, quat, s.vel, s.L)
        return m

    run = engine("mixed", "bussi")
    ref = engine("double", "no")
    sys.path.insert(0, os.path.join(HERE, "oracle"))
    import oracle
    p_or = oracle.make_params(oracle.make_settings(s.T, 0.5))
    f_max = t_max = 0.0
    f_num = f_den = t_num = t_den = 0.0
    f_rel, t_rel = [], []
    e_err = np.zeros(8)
    o_max = o_norm = 0.0
    for k in range(args.snapshots):
        run.run(args.every)
        st = run.get_state()
        F, T, E, Es = run.compute_forces()
        ref.set_state(st["pos"], st["quat"], st["vel"], st["Lmom"])
        Fr, Tr, Er, Esr = ref.compute_forces()
        n = np.linalg.norm(Fr, axis=1)
        fl = 0.1 * np.sqrt(np.mean(n ** 2))
        f_rel.append(np.linalg.norm(F - Fr, axis=1) / np.maximum(n, fl))
        f_max = max(f_max, float(np.max(f_rel[-1])))
        nt = np.linalg.norm(Tr, axis=1)
        tl = 0.1 * np.sqrt(np.mean(nt ** 2))
        t_rel.append(np.linalg.norm(T - Tr, axis=1) / np.maximum(nt, tl))
        t_max = max(t_max, float(np.max(t_rel[-1])))
        f_num += float(np.sum((F - Fr) ** 2)); f_den += float(np.sum(Fr ** 2))
        t_num += float(np.sum((T - Tr) ** 2)); t_den += float(np.sum(Tr ** 2))
        e_err = np.maximum(e_err, np.abs(Es - Esr) / abs(float(np.sum(Esr))))
        if k % max(1, args.snapshots // 5) == 0:
            f1, f2, f3 = oxio.quat_to_frame(st["quat"])
            rc, Fo, To, Eso, Epo = oracle.forces(p_or, st["pos"], f1, f2, f3, s.top.n3, s.top.n5, s.top.type, s.top.btype,
                                                 s.box, nthreads=cpu_cores())
            no = np.linalg.norm(Fo, axis=1)
            o_max = max(o_max, float(np.max(np.linalg.norm(F - Fo, axis=1) / np.maximum(no, 0.1 * np.sqrt(np.mean(no ** 2))))))
            o_norm = max(o_norm, float(np.linalg.norm(F - Fo) / np.linalg.norm(Fo)))
    run.close()
    ref.close()
    pct = [50, 99, 99.9, 99.99]
    f_pct = np.percentile(np.concatenate(f_rel), pct).tolist()
    t_pct = np.percentile(np.concatenate(t_rel), pct).tolist()

    drift = {}
    for precision in ("mixed", "float", "double"):
        m = engine(precision, "no")
        ts, es = [], []
        nsteps = args.nve_steps_double if precision == "double" else args.nve_steps
        for k in range(args.nve_samples + 1):
            if k:
                m.run(nsteps // args.nve_samples)
            U, Kt, Kr = m.energies()
            ts.append(k * (nsteps // args.nve_samples))
            es.append((U + Kt + Kr) / s.N)
        m.close()
        slope = float(np.polyfit(np.array(ts, float), np.array(es), 1)[0])
        drift[precision] = {"per_1e6_steps": slope * 1e6, "unit": "total energy per nucleotide (simulation units)",
                            "relative_per_1e6_steps": slope * 1e6 / abs(es[0]), "steps": ts[-1], "e0": es[0],
                            "e_end": es[-1]}
    line = {"study": "precision", "workload": "plain40k", "n_nucleotides": s.N, "snapshots": args.snapshots,
            "every": args.every,
            "mixed_vs_fp64_kernels": {"force_normwise": (f_num / f_den) ** 0.5, "force_max_per_particle": f_max,
                                      "torque_normwise": (t_num / t_den) ** 0.5, "torque_max_per_particle": t_max,
                                      "per_particle_percentiles": pct, "force_per_particle_at": f_pct,
                                      "torque_per_particle_at": t_pct,
                                      "energy_term_max_rel": e_err.tolist(),
                                      "energy_terms": ["FENE", "BEXC", "STCK", "NEXC", "HB", "CRST", "CXST", "DH"]},
            "mixed_vs_cpu_oracle": {"force_normwise_max": o_norm, "force_max_per_particle": o_max,
                                    "snapshots": len(range(0, args.snapshots, max(1, args.snapshots // 5)))},
            "per_particle_floor": "0.1 x RMS of the FP64 values",
            "nve_drift": drift}
    print(json.dumps(line), flush=True)


def averages_study(args):
    """Long-run averages of mixed precision against FP64 (the FP64 engine follows the
    reference's MD to 1e-8): independent Brownian runs of the same duplex system in both
    precisions; the potential, hydrogen-bonding and stacking energy per nucleotide, sampled every
    `every` steps, with standard errors from `blocks` block averages, and the z-score of each
    difference."""
    import torch
    torch.cuda.set_device(0)
    import oxdna_gb300 as ox
    from oxdna_gb300 import generate as G
    from oxdna_gb300 import io as oxio
    s = G.system_for_config(1, seed=args.seed, scale=args.avg_scale)
    a1, a2, a3 = s.frames()
    quat = oxio.frame_to_quat(a1, a2, a3)
    out = {}
    for precision in ("mixed", "double"):
        m = ox.MDSystem(s.box, s.top, ox.dna2_settings(s.T, 0.5),
                        ox.md_settings(dt=0.003, thermostat="john", newtonian_steps=103, diff_coeff=2.5,
                                       seed=101 if precision == "mixed" else 202, precision=precision,
                                       steps_per_graph=25))
        m.set_state(s.pos, quat, s.vel, s.L)
        m.run(args.avg_equil)
        rows = []
        for _ in range(args.avg_samples):
            m.run(args.every)
            _, _, _, Es = m.compute_forces()
            rows.append([Es.sum() / s.N, Es[4] / s.N, Es[2] / s.N])
        m.close()
        x = np.array(rows)
        b = x[: (len(x) // args.blocks) * args.blocks].reshape(args.blocks, -1, 3).mean(axis=1)
        out[precision] = (x.mean(axis=0), b.std(axis=0, ddof=1) / np.sqrt(args.blocks))
    names = ["potential", "hydrogen_bonding", "stacking"]
    res = {}
    for k, n in enumerate(names):
        (mm, sm), (md, sd) = (out["mixed"][0][k], out["mixed"][1][k]), (out["double"][0][k], out["double"][1][k])
        res[n] = {"mixed": mm, "mixed_se": sm, "double": md, "double_se": sd, "z": (mm - md) / np.hypot(sm, sd)}
    print(json.dumps({"study": "long-run averages", "workload": f"{s.N // 40} x 20-bp duplexes ({s.N} nt), 300 K, Brownian",
                      "unit": "energy per nucleotide (simulation units)", "equilibration_steps": args.avg_equil,
                      "samples": args.avg_samples, "every": args.every, "blocks": args.blocks, "averages": res}),
          flush=True)


def count_force_flops(ox, systems, offsets, st, nb_rows, nnb):
    """Algorithmic FLOPs of one force evaluation (every bond and every unordered pair once;
    oxgb_count_flops) summed over the systems of an engine, from the engine's own state and
    Verlet rows; returns (flops, sfu ops, pairs listed, pairs within the cutoff)."""
    from oxdna_gb300 import io as oxio
    tools = C.CDLL(ox.build.TOOLS)
    dp = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
    ip = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
    tools.oxgb_count_flops.argtypes = [C.c_int, dp, dp, dp, ip, ip, ip, ip, C.c_double, ip, ip, C.c_int, C.c_double,
                                       C.c_double, C.c_double, dp]
    fa1, _, fa3 = oxio.quat_to_frame(st["quat"])
    tot = np.zeros(4)
    for k, sy in enumerate(systems):
        o, n = int(offsets[k]), sy.N
        rows = np.ascontiguousarray(nb_rows[o:o + n] - o, np.int32)
        out = np.zeros(4)
        c = lambda a: np.ascontiguousarray(a[o:o + n])
        tools.oxgb_count_flops(n, c(st["pos"]), c(fa1), c(fa3), sy.top.n3, sy.top.n5, sy.top.type, sy.top.btype,
                               float(sy.box), rows.reshape(-1), np.ascontiguousarray(nnb[o:o + n]), rows.shape[1],
                               float(sy.T), 0.5, 0.05, out)
        tot += out
    return tot


def force_launch_seconds(L, _abi, sysm, stream, torch, reps=50):
    """CUDA-event time of one force evaluation with energies (oxgb_md_launch_forces: the
    bonded/pair and non-bonded kernels) on the engine's stream, current state"""
    with torch.cuda.stream(stream):
        for _ in range(3):
            _abi.check(L.oxgb_md_launch_forces(sysm.handle))
        f0 = torch.cuda.Event(enable_timing=True)
        f1 = torch.cuda.Event(enable_timing=True)
        f0.record(stream)
        for _ in range(reps):
            _abi.check(L.oxgb_md_launch_forces(sysm.handle))
        f1.record(stream)
    torch.cuda.synchronize()
    return f0.elapsed_time(f1) * 1e-3 / reps


def roofline_of(ox, L, _abi, sysm, stream, torch, systems, peak, traffic=None):
    st = sysm.get_state()
    nnb, nb, _, _ = sysm.neighbours()
    flops, sfu, pairs, in_range = count_force_flops(ox, systems, sysm.offsets, st, nb, nnb)
    t_force = force_launch_seconds(L, _abi, sysm, stream, torch)
    achieved = flops / t_force
    return {"bound": "fp32", "achieved": achieved / 1e12, "peak": peak / 1e12, "unit": "TFLOP/s",
            "frac": achieved / peak, "traffic": traffic,
            "traffic_note": "DRAM bytes (read + write) of one launch of the two force kernels, from an ncu "
                            "--set full capture with cold caches; the timed launches find their data in L2",
            "kernel": "k_bonded_pairs + k_nonbonded_split (FP32 pair math)",
            "flops_per_launch": flops, "sfu_per_launch": sfu, "launch_ms": t_force * 1e3,
            "unordered_pairs_listed": pairs, "unordered_pairs_in_cutoff": in_range,
            "flop_count": "every bond and every unordered pair once (partner torque included), "
                          "term branches actually taken; counted by csrc/flopcount.cpp on this state",
            "peak_source": "FP32 FMA throughput measured on this GPU by oxgb_probe_fp32_peak "
                           "(MEASURED_PEAKS.json has HBM and bf16 peaks only)"}


def force_error(sysm, s, st):
    sys.path.insert(0, os.path.join(HERE, "oracle"))
    import oracle
    from oxdna_gb300 import io as oxio
    F, T, E, Es = sysm.compute_forces()
    fa1, fa2, fa3 = oxio.quat_to_frame(st["quat"])
    p = oracle.make_params(oracle.make_settings(s.T, 0.5))
    rc, Fo, To, Eso, Epo = oracle.forces(p, st["pos"], fa1, fa2, fa3, s.top.n3, s.top.n5, s.top.type, s.top.btype,
                                         s.box, nthreads=cpu_cores())
    n = np.linalg.norm(Fo, axis=1)
    floor = 0.1 * np.sqrt(np.mean(n ** 2))
    den = np.maximum(n, floor)
    rel = np.linalg.norm(F - Fo, axis=1) / den
    # the oracle's own response to the axes rounded to FP32 (the input the mixed path rounds)
    r1, r3 = fa1.astype(np.float32).astype(np.float64), fa3.astype(np.float32).astype(np.float64)
    _, Fr, _, _, _ = oracle.forces(p, st["pos"], r1, np.cross(r3, r1), r3, s.top.n3, s.top.n5, s.top.type,
                                   s.top.btype, s.box, nthreads=cpu_cores())
    bound = np.linalg.norm(F - Fo, axis=1) / (1e-5 * den + 2 * np.linalg.norm(Fr - Fo, axis=1))
    return {"normwise": float(np.linalg.norm(F - Fo) / np.linalg.norm(Fo)),
            "max_per_particle": float(np.max(rel)),
            "per_particle_p99_99": float(np.percentile(rel, 99.99)),
            "per_particle_over_1e-5": int((rel > 1e-5).sum()),
            "max_of_conditioning_bound": float(np.max(bound)),
            "conditioning_bound": "|dF_i| <= 1e-5 max(|F_i|, floor) + 2 |F_i(FP32 axes) - F_i|, FP64 oracle",
            "per_particle_floor": "0.1 x RMS |F| of the FP64 oracle",
            "torque_normwise": float(np.linalg.norm(T - To) / np.linalg.norm(To)),
            "energy_rel": float(abs(Es.sum() - Eso.sum()) / abs(Eso.sum())),
            "oracle": "FP64 CPU restatement of DNA2_nomesh (oracle/), pinned to the reference"}


def plain_run(args, name, rank, world, torch, ox, _abi, peak):
    """One system (a replica per rank) through the plain path: `value` on HBM-resident state,
    the roofline of its force kernels and (headline, rank 0) the force error against the FP64
    oracle and the end-to-end figure through the C ABI with host buffers."""
    from oxdna_gb300 import io as oxio
    wl = WORKLOADS[name]
    s = relax(make_system(wl, args.seed + rank), wl, args.seed + rank)
    a1, a2, a3 = s.frames()
    quat = oxio.frame_to_quat(a1, a2, a3)
    sort_every = wl.get("sort_every", 0) if args.sort_every is None else args.sort_every
    md = ox.md_settings(dt=wl["dt"], thermostat=wl["thermostat"], newtonian_steps=wl["newtonian_steps"],
                        bussi_tau=wl.get("bussi_tau", 1000.0), diff_coeff=wl.get("diff_coeff", 2.5), seed=1 + rank,
                        precision="mixed", steps_per_graph=25, list_rebuild_node=args.list_node,
                        sort_every=sort_every, autotune=not args.no_autotune and args.force_shape is None,
                        use_edge=args.use_edge, list_kernel=args.list_kernel)
    sysm = ox.MDSystem(s.box, s.top, ox.dna2_settings(s.T, 0.5), md)
    sysm.set_state(s.pos, quat, s.vel, s.L)
    if args.force_shape is not None:
        sysm.set_force_shape(args.force_shape)
    shape = sysm.force_shape()
    L = _abi.lib()
    stream = torch.cuda.ExternalStream(sysm.stream)
    M = args.md_steps
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")  # 256 MiB > L2

    for _ in range(args.warmup):
        sysm.run(M, sync=False)
    torch.cuda.synchronize()
    _abi.check(L.oxgb_md_status(sysm.handle))
    info0 = sysm.info()
    if world > 1:
        torch.distributed.barrier()
    clocks = ClockSampler(int(os.environ.get("LOCAL_RANK", "0")))
    clocks.start()
    times = []
    with torch.cuda.stream(stream):
        for k in range(args.steps):
            flush.fill_(float(k))
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            sysm.run(M, sync=False)
            e1.record(stream)
            times.append((e0, e1))
    torch.cuda.synchronize()
    clk = clocks.stop()
    if world > 1:
        torch.distributed.barrier()
    _abi.check(L.oxgb_md_status(sysm.handle))
    info1 = sysm.info()
    t_dev = sum(a.elapsed_time(b) for a, b in times) * 1e-3
    if world > 1:
        tt = torch.tensor([t_dev], device="cuda")
        torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
        t_dev = float(tt.item())
    steps_total = args.steps * M
    rebuilds = info1["rebuilds"] - info0["rebuilds"]
    out = {"value": world * s.N * steps_total / t_dev, "unit": "particle-steps/s", "ms_per_step": t_dev / args.steps * 1e3,
           "n_nucleotides": s.N, "md_steps_per_step": M, "md_steps_per_s": steps_total / t_dev,
           "list_rebuilds": rebuilds, "clocks": clk, "description": wl["desc"], "force_shape": shape,
           "use_edge": bool(args.use_edge)}
    out["roofline"] = roofline_of(ox, L, _abi, sysm, stream, torch, [s], peak, FORCE_TRAFFIC.get(name))
    st = sysm.get_state()
    if rank == 0 and not args.no_cpu_baseline:
        out["force_error_vs_fp64"] = force_error(sysm, s, st)
    if not args.no_e2e:
        host = dict(pos=np.ascontiguousarray(st["pos"]), quat=np.ascontiguousarray(st["quat"]),
                    vel=np.ascontiguousarray(st["vel"]), L=np.ascontiguousarray(st["Lmom"]))
        ne = max(1, min(args.steps, 5))
        got = sysm.get_state()  # the host arrays the loop reads the state back into
        # one untimed round first, as the warm-up steps before `value`: an upload after the timed
        # steps may size the term lists up (their longest rows grew) and capture the step graph again
        sysm.set_state(host["pos"], host["quat"], host["vel"], host["L"])
        sysm.run(M, sync=True)
        got = sysm.get_state(out=got)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(ne):
            sysm.set_state(host["pos"], host["quat"], host["vel"], host["L"])
            sysm.run(M, sync=True)
            got = sysm.get_state(out=got)
        t_e2e = time.perf_counter() - t0
        h2d = s.N * (3 + 4 + 3 + 3) * 8
        out["e2e"] = {"value": world * s.N * M * ne / t_e2e, "unit": "particle-steps/s", "h2d_bytes_per_step": h2d,
                      "d2h_bytes_per_step": h2d, "md_steps_per_step": M,
                      "what": "per step: oxgb_md_set_state from host arrays (upload, list build, forces), M MD "
                              "steps, oxgb_md_get_state into the same host arrays every step; wall clock"}
        assert np.all(np.isfinite(got["pos"]))
    # our kernels in the timed region: per MD step the first step, the bonded + pair kernel and
    # the non-bonded kernel, the Bussi draws and sums (the last block of a system makes its
    # update), and either the rebuild condition (conditional node: 10 list kernels per rebuild)
    # or the 10 list kernels themselves (kernel node: they return at once unless a system is
    # stale); per graph of 25 steps the step advance; per run the 2-kernel flush
    per_step = 3 + (2 if wl["thermostat"] == "bussi" else 0)
    if args.list_node == "conditional":
        per_step += 1
        list_launches = rebuilds * 10
    else:
        per_step += 10
        list_launches = 0
    out["gpu_launches"] = int(steps_total * per_step + list_launches + (steps_total // 25) + 2 * args.steps)
    out["_system"] = s
    sysm.close()
    return out


def batched_roofline(args, ox, _abi, torch, peak):
    """roofline of the force kernels of the 256-system engine (same FLOP count, per system)"""
    from oxdna_gb300 import io as oxio
    systems = batched_workload(args.seed)
    b = ox.MDSystem([x.box for x in systems], [x.top for x in systems], [ox.dna2_settings(x.T, 0.5) for x in systems],
                    ox.md_settings(dt=0.003, thermostat="bussi", newtonian_steps=1, bussi_tau=1000.0, seed=7,
                                   precision="mixed", steps_per_graph=25, autotune=not args.no_autotune))

    def state(x):
        a1, a2, a3 = x.frames()
        return x.pos, oxio.frame_to_quat(a1, a2, a3), x.vel, x.L

    b.set_state(*[np.concatenate(v) for v in zip(*[state(x) for x in systems])])
    b.run(args.md_steps)
    L = _abi.lib()
    stream = torch.cuda.ExternalStream(b.stream)
    r = roofline_of(ox, L, _abi, b, stream, torch, systems, peak, None)
    b.close()
    return r


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference", "reference-cuda"])
    ap.add_argument("--workload", default="large250k", choices=sorted(WORKLOADS))
    ap.add_argument("--also", default="plain40k", help="comma-separated workloads reported as sub-objects ('' for none)")
    ap.add_argument("--md-steps", type=int, default=200, help="MD steps per timed iteration")
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--cpu-sample-steps", type=int, default=2, help="MD steps of the FP64 oracle port's sample")
    ap.add_argument("--cpu-steps", type=int, default=5, help="MD steps of each reference CPU copy")
    ap.add_argument("--reference-repeats", type=int, default=1,
                    help="--impl reference: timed samples (each a run of every copy)")
    ap.add_argument("--ref-cuda-steps", type=int, nargs=2, default=None,
                    help="--impl reference-cuda: step counts of its two runs (default 1000 and "
                         "1000 + max(5000, 2e9 / N))")
    ap.add_argument("--ref-cuda-energy", action="store_true",
                    help="--impl reference-cuda: also compare its device energy with ours")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--port-baseline", action="store_true", help="time the FP64 oracle port as the CPU baseline")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-autotune", action="store_true", help="default force-kernel shape instead of the autotuned one")
    ap.add_argument("--force-shape", type=int, default=None,
                    help="pin force-kernel shape k of the autotuner's table instead of tuning (profiling)")
    ap.add_argument("--list-kernel", default="auto", choices=["auto", "warp", "thread", "group4", "group8", "group16"],
                    help="neighbour-row kernel of the list build (auto: the autotuner's choice)")
    ap.add_argument("--use-edge", action="store_true",
                    help="use_edge: Debye-Hueckel and excluded volume once per pair with atomic adds (A/B variant)")
    ap.add_argument("--no-batched", action="store_true", help="skip the 256-system batched workload")
    ap.add_argument("--batched-only", action="store_true",
                    help="only the batched engine (no plain workloads, no one-at-a-time comparison): profiling")
    ap.add_argument("--list-node", default="conditional", choices=["conditional", "kernel"],
                    help="list rebuild as a conditional graph node, or as always-launched kernels that "
                         "return at once on a fresh list (what a kernel-level profiler can see)")
    ap.add_argument("--sort-every", type=int, default=None,
                    help="store nucleotides in cell order every k-th list rebuild (default: the workload's)")
    ap.add_argument("--precision-study", action="store_true",
                    help="instead of the throughput line: force/torque/energy errors over snapshots and NVE drift")
    ap.add_argument("--averages-study", action="store_true",
                    help="instead of the throughput line: long-run energy averages, mixed vs FP64")
    ap.add_argument("--avg-scale", type=float, default=0.05, help="duplex count of the averages study / 1000")
    ap.add_argument("--avg-equil", type=int, default=20000)
    ap.add_argument("--avg-samples", type=int, default=400)
    ap.add_argument("--blocks", type=int, default=20)
    ap.add_argument("--snapshots", type=int, default=100)
    ap.add_argument("--every", type=int, default=1000)
    ap.add_argument("--nve-steps", type=int, default=100000)
    ap.add_argument("--nve-steps-double", type=int, default=20000)
    ap.add_argument("--nve-samples", type=int, default=20)
    args = ap.parse_args()
    if args.precision_study:
        precision_study(args)
        return
    if args.averages_study:
        averages_study(args)
        return
    if args.warmup < 3:
        args.warmup = 3
    wl = WORKLOADS[args.workload]
    if args.impl == "reference":
        run_reference_arm(args, wl)
        return
    if args.impl == "reference-cuda":
        run_reference_cuda_arm(args, wl)
        return

    import torch
    rank, world, local = env_rank()
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    else:
        torch.cuda.set_device(0)

    import oxdna_gb300 as ox
    from oxdna_gb300 import _abi
    L = _abi.lib()
    peak = C.c_double(0)
    _abi.check(L.oxgb_probe_fp32_peak(C.byref(peak)))

    if args.batched_only:
        print(json.dumps(bench_batched(args, torch, ox, _abi, compare=False)))
        return
    head = plain_run(args, args.workload, rank, world, torch, ox, _abi, peak.value)
    s = head.pop("_system")
    subs = {}
    for name in [w for w in args.also.split(",") if w and w != args.workload]:
        sub = plain_run(args, name, rank, world, torch, ox, _abi, peak.value)
        sub.pop("_system")
        subs[name] = sub
    line_extra = {}
    if not args.no_batched:
        if world == 1:
            bt = bench_batched(args, torch, ox, _abi)
            bt["roofline"] = batched_roofline(args, ox, _abi, torch, peak.value)
            line_extra["batched"] = bt
        else:
            line_extra["batched"] = bench_batched_sharded(args, torch, ox, _abi, rank, world)
    if rank == 0 and not args.no_cpu_baseline:
        cpu = None if args.port_baseline else reference_cpu_baseline(make_system(wl, args.seed), wl, args.seed,
                                                                      args.cpu_steps)
        line_extra["cpu_baseline"] = cpu or port_cpu_baseline(s, wl, args.cpu_sample_steps)

    line = {
        "metric": "oxDNA2 MD particle-steps/s", "value": head["value"], "unit": "particle-steps/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": head["ms_per_step"],
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": args.workload, "n_nucleotides": head["n_nucleotides"], "description": wl["desc"],
                   "md_steps_per_step": args.md_steps,
                   "l2": "flushed before every timed iteration (256 MiB write)", "precision": "FP32 forces, FP64 state",
                   "parallelism": "replicas" if world > 1 else "single GPU",
                   "sort_every": wl.get("sort_every", 0) if args.sort_every is None else args.sort_every,
                   "force_shape": head["force_shape"], "use_edge": bool(args.use_edge)},
        "md_steps_per_s": head["md_steps_per_s"],
        "list_rebuilds": head["list_rebuilds"],
        "roofline": head["roofline"],
        "clocks": head["clocks"],
        "e2e": head.get("e2e"),
        "gpu_launches": head["gpu_launches"],
    }
    if "force_error_vs_fp64" in head:
        line["force_error_vs_fp64"] = head["force_error_vs_fp64"]
    for name, sub in subs.items():
        line[name] = sub
    line.update(line_extra)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
