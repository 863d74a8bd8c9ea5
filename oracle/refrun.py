"""Runs the reference oxDNA programs on systems generated here, and times them.

BASELINE / CHECKER infrastructure, not product code: only bench.py's reference arms and tests
use this module.  The programs are the reference's own, built from its own sources by
oracle/ref/Makefile (no CMake) into oracle/_ref/:

  * oxDNA_cpu  -- the Release CPU program (-O3 -ffast-math, double precision), single-threaded
    by design (one system per process);
  * oxDNA_cuda -- the Release program with the CUDA backend (backend = CUDA, the default
    backend_precision = mixed, CUDA_list = verlet), compiled for sm_103a.

The reference checkout is the folder OXDNA_REFERENCE names or, on a machine without it, the copy
that `make -C oracle/ref stage` leaves (untracked) in baseline/_ref/oxDNA.

Steps are timed without the program's set-up.  A GPU run (time_steps) runs the same deck twice,
with `steps_a` and `steps_b` steps, and divides the difference of the two wall times by the
difference of the step counts (set-up, reading the configuration and the first list build
cancel).  CPU copies (cpu_rates) are timed by the program's own timer of its step loop ("Total
Running Time ... per step", CPU clock), which leaves the set-up out.
"""

from __future__ import annotations

import os
import re
import subprocess
import tempfile
import time
from typing import Optional

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
OUT = os.path.join(HERE, "_ref")
PROGRAMS = {"cpu": os.path.join(OUT, "oxDNA_cpu"), "cuda": os.path.join(OUT, "oxDNA_cuda"),
            "cuda-gb300": os.path.join(OUT, "oxDNA_cuda_gb300"), "plugin": os.path.join(OUT, "plugins", "CUDAGB300DNA2.so")}


def reference_checkout() -> Optional[str]:
    """the oxDNA checkout to build from, or None"""
    for cand in (os.environ.get("OXDNA_REFERENCE", ""), os.path.join(REPO, "baseline", "_ref", "oxDNA")):
        if cand and os.path.isfile(os.path.join(cand, "src", "oxDNA.cpp")):
            return cand
    return None


def build(kind: str, jobs: Optional[int] = None, log: Optional[str] = None) -> str:
    """builds a reference program (kind: cpu, cuda, or cuda-gb300 -- the CUDA program with our
    interaction and Verlet list linked in under the reference's class names) or the plugin
    (plugin) if it is missing; returns its path"""
    exe = PROGRAMS[kind]
    if os.path.exists(exe):
        return exe
    ref = reference_checkout()
    if ref is None:
        raise FileNotFoundError("no oxDNA reference sources (set OXDNA_REFERENCE or stage them in baseline/_ref/oxDNA)")
    jobs = jobs or (len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else (os.cpu_count() or 4))
    fh = open(log, "w") if log else subprocess.DEVNULL
    try:
        r = subprocess.run(["make", "-s", "-C", os.path.join(HERE, "ref"), f"-j{jobs}", f"REF={ref}", kind],
                           stdout=fh, stderr=subprocess.STDOUT)
    finally:
        if log:
            fh.close()
    if r.returncode != 0 or not os.path.exists(exe):
        raise RuntimeError(f"building the reference {kind} program failed (make exit {r.returncode})")
    return exe


def deck(s, *, backend: str, steps: int, dt: float, thermostat: str = "no", newtonian_steps: int = 103,
         diff_coeff: float = 2.5, bussi_tau: float = 1000.0, seed: int = 1, salt: float = 0.5,
         interaction: str = "DNA2", skin: float = 0.05, print_every: int = 0, extra: str = "") -> str:
    """the input file of one run of system `s` (topology init.top, configuration init.dat, in the
    run's folder); nothing is printed inside the step loop unless print_every asks for energies,
    the last configuration is written after it"""
    lines = [
        f"backend = {backend}",
        "sim_type = MD",
        f"interaction_type = {interaction}",
        f"salt_concentration = {salt!r}",
        f"T = {s.T!r}",
        f"dt = {dt!r}",
        f"steps = {int(steps)}",
        f"seed = {int(seed)}",
        f"verlet_skin = {skin!r}",
        f"thermostat = {thermostat}",
        f"newtonian_steps = {int(newtonian_steps)}",
        f"diff_coeff = {diff_coeff!r}",
        f"bussi_tau = {bussi_tau!r}",
        "topology = init.top",
        "conf_file = init.dat",
        "trajectory_file = trajectory.dat",
        "lastconf_file = last_conf.dat",
        "energy_file = energy.dat",
        "refresh_vel = 0",
        "restart_step_counter = 1",
        "no_stdout_energy = 0",
        "time_scale = linear",
        "print_conf_interval = 1000000000",
        f"print_energy_every = {int(print_every) if print_every > 0 else 1000000000}",
        "external_forces = 0",
    ]
    if backend == "CUDA":
        lines += ["backend_precision = mixed", "CUDA_list = verlet", "CUDA_sort_every = 0",
                  "CUDA_avoid_cpu_calculations = true"]
    return "\n".join(lines) + "\n" + extra


def write_system(folder: str, s) -> None:
    s.write(os.path.join(folder, "init.top"), os.path.join(folder, "init.dat"))


_PER_STEP = re.compile(r"Total Running Time:\s*([0-9.eE+-]+)\s*s,\s*per step:\s*([0-9.eE+-]+)\s*ms")


def run(exe: str, folder: str, text: str, timeout: float = 1800.0, tag: str = "input") -> dict:
    """runs the program on the deck `text` in `folder`; returns wall time, the program's own
    per-step figure and its output"""
    path = os.path.join(folder, tag)
    with open(path, "w") as fh:
        fh.write(text)
    t0 = time.perf_counter()
    r = subprocess.run([exe, tag], cwd=folder, capture_output=True, text=True, timeout=timeout)
    wall = time.perf_counter() - t0
    out = r.stdout + r.stderr
    if r.returncode != 0:
        raise RuntimeError(f"{os.path.basename(exe)} failed (exit {r.returncode}):\n{out[-3000:]}")
    m = _PER_STEP.search(out)
    return {"wall_s": wall, "own_total_s": float(m.group(1)) if m else None,
            "own_ms_per_step": float(m.group(2)) if m else None, "log": out}


def time_steps(exe: str, s, steps_a: int, steps_b: int, folder: Optional[str] = None, **deck_kw) -> dict:
    """seconds per step of the program on system s, from two runs of steps_a < steps_b steps"""
    own = folder is None
    tmp = tempfile.mkdtemp(prefix="oxref_") if own else folder
    write_system(tmp, s)
    ra = run(exe, tmp, deck(s, steps=steps_a, **deck_kw), tag="input_a")
    rb = run(exe, tmp, deck(s, steps=steps_b, **deck_kw), tag="input_b")
    per = (rb["wall_s"] - ra["wall_s"]) / (steps_b - steps_a)
    return {"s_per_step": per, "steps": (steps_a, steps_b), "wall_s": (ra["wall_s"], rb["wall_s"]),
            "own_ms_per_step": rb["own_ms_per_step"], "folder": tmp, "log_b": rb["log"][-4000:]}


_CUDA_E = re.compile(r"CUDA_energy:\s*([-0-9.eE+]+)")


def cuda_energy_per_nucleotide(exe: str, s, folder: Optional[str] = None, salt: float = 0.5, interaction: str = "DNA2",
                               extra: str = "") -> float:
    """the potential energy per nucleotide that the reference CUDA backend computes on the
    device (CUDA_print_energy) for the configuration of s: three steps with a vanishing time step
    and no thermostat, so the state does not move; the value printed after the first step"""
    tmp = folder or tempfile.mkdtemp(prefix="oxref_e_")
    write_system(tmp, s)
    # the backend_info observable prints the string CUDA_print_energy fills in each step
    extra = extra + ("CUDA_print_energy = true\n"
                     "data_output_1 = {\n  name = backend_info.dat\n  print_every = 1\n  col_1 = {\n"
                     "    type = backend_info\n  }\n}\n")
    text = deck(s, backend="CUDA", steps=3, dt=1e-12, salt=salt, print_every=1, interaction=interaction, extra=extra)
    r = run(exe, tmp, text, tag="input_e")
    info = open(os.path.join(tmp, "backend_info.dat")).read() if os.path.exists(os.path.join(tmp, "backend_info.dat")) else ""
    vals = [float(v) for v in _CUDA_E.findall(info + r["log"])]
    if not vals:
        raise RuntimeError("no CUDA_energy in the reference output:\n" + info[-1000:] + r["log"][-2000:])
    return vals[0]


def cpu_batch_rate(exe: str, systems, n_proc: int, steps: int, **deck_kw) -> dict:
    """The reference CPU program on every system of a batch (each with its own temperature),
    n_proc processes at a time, one per core, `steps` MD steps each timed by the program's own
    step-loop timer.  The batch's throughput on n_proc cores with perfect packing: sum N_i /
    (sum t_i / n_proc), t_i the seconds per step of system i."""
    import concurrent.futures as cf
    tmp = tempfile.mkdtemp(prefix="oxref_batch_")

    def one(k):
        s = systems[k]
        d = os.path.join(tmp, f"s{k}")
        os.makedirs(d, exist_ok=True)
        write_system(d, s)
        r = run(exe, d, deck(s, steps=steps, seed=1 + k, **deck_kw), tag="input")
        if r["own_ms_per_step"] is None:
            raise RuntimeError(f"no step timer in the output of system {k}")
        return r["own_ms_per_step"] * 1e-3

    t0 = time.perf_counter()
    with cf.ThreadPoolExecutor(max_workers=n_proc) as ex:
        per = list(ex.map(one, range(len(systems))))
    wall = time.perf_counter() - t0
    n_tot = sum(s.N for s in systems)
    return {"value": n_tot / (sum(per) / n_proc), "s_per_step_sum": sum(per), "wall_s": wall}


def reference_verlet_list(exe: str, plugin_dir: str, s, salt: float = 0.5) -> dict:
    """the first Verlet list the reference CUDA backend builds for system s with its own
    CUDASimpleVerletList (CUDA_list = verlet), as handed to the GB300DNA2 plugin, which writes it
    (key gb300_dump_list) with the FP32 positions it was built from: counts[N], the column-major
    rows and pos[N, 4]"""
    tmp = tempfile.mkdtemp(prefix="oxref_list_")
    write_system(tmp, s)
    dump = os.path.join(tmp, "list.bin")
    extra = f"plugin_search_path = {plugin_dir}\ngb300_dump_list = {dump}\n"
    run(exe, tmp, deck(s, backend="CUDA", steps=1, dt=1e-12, salt=salt, interaction="GB300DNA2", extra=extra),
        tag="input_list")
    raw = np.fromfile(dump, dtype=np.int32)
    N, maxc = int(raw[0]), int(raw[1])
    counts = raw[2:2 + N].copy()
    rows = raw[2 + N:2 + N + maxc * N].reshape(maxc, N).T.copy()
    pos = raw[2 + N + maxc * N:2 + N + maxc * N + 4 * N].view(np.float32).reshape(N, 4).copy()
    return {"counts": counts, "rows": rows, "pos": pos}


def cpu_rates(exe: str, s, n_proc: int, steps: int, **deck_kw) -> dict:
    """n_proc independent copies of the single-threaded CPU program on system s, run at the same
    time, one per core; each copy's seconds per step come from its own timer of the step loop
    ("Total Running Time ... per step", CPU clock, set-up excluded).  Returns the summed
    particle-steps/s."""
    tmp = tempfile.mkdtemp(prefix="oxref_cpu_")
    write_system(tmp, s)
    procs = []
    t0 = time.perf_counter()
    for k in range(n_proc):
        d = os.path.join(tmp, f"r{k}")
        os.makedirs(d, exist_ok=True)
        for f in ("init.top", "init.dat"):
            os.link(os.path.join(tmp, f), os.path.join(d, f))
        with open(os.path.join(d, "input"), "w") as fh:
            fh.write(deck(s, steps=steps, seed=1 + k, **deck_kw))
        log = open(os.path.join(d, "log.txt"), "w")
        procs.append((subprocess.Popen([exe, "input"], cwd=d, stdout=log, stderr=subprocess.STDOUT), log, d))
    per = []
    for p, log, d in procs:
        rc = p.wait()
        log.close()
        text = open(os.path.join(d, "log.txt")).read()
        m = _PER_STEP.search(text)
        if rc != 0 or m is None:
            raise RuntimeError(f"reference CPU copy in {d} failed (exit {rc}):\n{text[-2000:]}")
        per.append(float(m.group(2)) * 1e-3)
    wall = time.perf_counter() - t0
    per = np.array(per)
    return {"value": float(np.sum(s.N / per)), "s_per_step": float(np.mean(per)), "s_per_step_max": float(np.max(per)),
            "processes": n_proc, "steps": steps, "wall_s": wall}


def read_last_conf(folder: str):
    from oxdna_gb300 import io as oxio
    return oxio.read_conf(os.path.join(folder, "last_conf.dat"))


def pos_array(conf) -> np.ndarray:
    return np.asarray(conf.pos)
