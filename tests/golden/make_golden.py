"""Generate the golden fixtures that pin the oracle (and through it the GPU kernels) to the
reference implementation.

Each fixture is produced by running the reference oxDNA CPU code, built from its own sources
by oracle/ref/Makefile into oracle/_ref/ref_dump, on a small input deck: the reference reads the
topology and configuration, and the harness prints its internal state, full-precision forces,
torques and energy split (interaction_type = DNA2_nomesh, the exact-f4 oxDNA2 force field).
Cases that ask for steps also record the state after a short reference MD run.

    make -C oracle/ref -j8 REF=$OXDNA_REFERENCE      # once
    python tests/golden/make_golden.py --ref $OXDNA_REFERENCE

The .npz files are small (tens of KB) and committed; tests never need the reference itself.
"""

from __future__ import annotations

import argparse
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

from oxdna_gb300 import generate as G  # noqa: E402
from oxdna_gb300 import io as oxio  # noqa: E402

DUMP = os.path.join(REPO, "oracle", "_ref", "ref_dump")


def parse_dump(path):
    lines = open(path).read().split("\n")
    d = {}
    i = 0
    while i < len(lines):
        ln = lines[i].split()
        if not ln:
            i += 1
            continue
        k = ln[0]
        if k == "box":
            d["box"] = np.array(list(map(float, ln[1:4])))
            i += 1
        elif k == "rcut":
            d["rcut"] = float(ln[1])
            i += 1
        elif k in ("topology", "state", "forces", "final"):
            n = int(ln[1])
            d[k] = np.array([list(map(float, lines[i + 1 + j].split())) for j in range(n)])
            i += n + 1
        elif k == "energy":
            d["energy"] = float(ln[1])
            i += 1
        elif k == "step":
            d["step"] = int(ln[1])
            i += 1
        elif k == "split":
            n = int(ln[1])
            d["split"] = np.array([float(lines[i + 1 + j].split()[1]) for j in range(n)])
            i += n + 1
        else:
            i += 1
    return d


BASE_INPUT = """backend = CPU
sim_type = MD
interaction_type = DNA2_nomesh
seed = 1
steps = {steps}
dt = {dt}
T = {T}
salt_concentration = {salt}
verlet_skin = 0.05
thermostat = no
newtonian_steps = 103
diff_coeff = 2.5
topology = init.top
conf_file = init.dat
trajectory_file = trajectory.dat
lastconf_file = last_conf.dat
energy_file = energy.dat
refresh_vel = 0
restart_step_counter = 1
no_stdout_energy = 1
time_scale = linear
print_conf_interval = 100000
print_energy_every = 100000
external_forces = 0
"""


def run_case(name, top_path, conf_path, settings, extra="", steps=0, dt=0.003):
    with tempfile.TemporaryDirectory() as tmp:
        open(os.path.join(tmp, "init.top"), "w").write(open(top_path).read())
        open(os.path.join(tmp, "init.dat"), "w").write(open(conf_path).read())
        text = BASE_INPUT.format(steps=steps, dt=dt, T=settings["T_str"], salt=settings["salt"]) + extra
        open(os.path.join(tmp, "input"), "w").write(text)
        out = os.path.join(tmp, "dump.txt")
        subprocess.run([DUMP, "input", out], cwd=tmp, check=True, stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
        d = parse_dump(out)
    top = d["topology"].astype(np.int64)
    st = d["state"]
    rec = dict(
        box=d["box"][0], rcut=d["rcut"], T=oxio.get_temperature(settings["T_str"]), salt=float(settings["salt"]),
        n3=top[:, 0].astype(np.int32), n5=top[:, 1].astype(np.int32), type=top[:, 2].astype(np.int32),
        btype=top[:, 3].astype(np.int32), pos=st[:, 0:3], a1=st[:, 3:6], a2=st[:, 6:9], a3=st[:, 9:12],
        vel=st[:, 12:15], Lmom=st[:, 15:18], F=d["forces"][:, 0:3], Tq=d["forces"][:, 3:6], split=d["split"],
        energy=d["energy"], average=int(settings.get("average", 1)),
        hb_multiplier=float(settings.get("hb_multiplier", 1.0)),
        half_charged_ends=int(settings.get("half_charged_ends", 1)),
        dh_lambda=float(settings.get("dh_lambda", 0.3616455)), dh_strength=float(settings.get("dh_strength", 0.0543)),
        mbf_fmax=float(settings.get("mbf_fmax", -1.0)), mbf_finf=float(settings.get("mbf_finf", 0.04)),
        steps=steps, dt=dt)
    if "seq" in settings:
        order = "AGCT"
        rec["seq_stck"] = np.array([[settings["seq"][f"STCK_{order[i]}_{order[j]}"] for j in range(4)] for i in range(4)])
        rec["seq_fact"] = settings["seq"]["STCK_FACT_EPS"]
        rec["seq_hydr_at"] = settings["seq"].get("HYDR_A_T", settings["seq"].get("HYDR_T_A"))
        rec["seq_hydr_gc"] = settings["seq"].get("HYDR_G_C", settings["seq"].get("HYDR_C_G"))
    if "final" in d:
        fs = d["final"]
        rec.update(final_pos=fs[:, 0:3], final_a1=fs[:, 3:6], final_a2=fs[:, 6:9], final_a3=fs[:, 9:12],
                   final_vel=fs[:, 12:15], final_Lmom=fs[:, 15:18])
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **rec)
    print(f"{name}: N={top.shape[0]} E={d['energy']:.6f} max|F|={np.abs(rec['F']).max():.3f}")


# the external forces of the ext_forces fixture, as the dicts MDSystem.set_external_forces and
# oracle.external_forces take, and as the reference's external_forces_file records
# (src/Forces/{ConstantRateForce,MutualTrap,MovingTrap,LowdimMovingTrap,RepulsionPlane,
# AttractionPlane,RepulsiveSphere,RepulsiveSphereSmooth,LJWall,GenericCentralForce,
# RepulsionPlaneMoving,LJCone}.cpp): twelve types, rates, a periodic mutual trap; the geometric
# parameters are placed relative to the configuration pos so that every record acts
def ext_force_set(N, box, pos):
    com = pos.mean(axis=0)
    zmin = float(pos[:, 2].min())
    u = np.array([0.48, -0.6, 0.64])
    return [
        dict(type="string", particle=0, F0=0.3, rate=1e-3, dir=(0.0, 0.6, 0.8)),
        dict(type="string", particle=5, F0=0.2, rate=0.0, dir=(1.0, 2.0, 3.0), dir_as_centre=True),
        dict(type="mutual_trap", particle=2, ref_particle=N - 3, stiff=0.9, r0=1.2, rate=2e-3, stiff_rate=1e-3),
        dict(type="mutual_trap", particle=N - 3, ref_particle=2, stiff=0.9, r0=0.5, PBC=True),
        dict(type="trap", particle=7, stiff=1.5, pos0=(1.0, -2.0, 0.5), rate=1e-2, dir=(0.0, 0.0, 1.0)),
        dict(type="lowdim_trap", particle=7, stiff=0.7, pos0=(0.5, 0.0, -0.5), rate=3e-3, dir=(1.0, 0.0, 0.0),
             visibility=(True, False, True)),
        dict(type="repulsion_plane", particle=9, stiff=2.0, dir=(0.0, 0.0, 1.0), position=box,
             r0=-(float(pos[:, 2].max()) + 1.0), rate=-0.05),
        dict(type="attraction_plane", particle=11, stiff=0.4, dir=(1.0, 0.0, 0.0), position=-1.0),
        dict(type="sphere", particle=13, stiff=0.8, r0=0.2, rate=1e-4, center=tuple(com)),
        dict(type="sphere", particle=1, stiff=0.8, r0=0.2, rate=1e-4, r_ext=30.0, center=tuple(com + box)),
        dict(type="sphere_smooth", particle=14, stiff=0.3, r0=0.1, r_ext=30.0, smooth=30.0, alpha=30.0,
             center=tuple(com)),
        dict(type="LJ_wall", particle=15, stiff=1.0, sigma=1.0, n=6, dir=(0.0, 0.0, 1.0), position=1.0 - zmin),
        dict(type="LJ_wall", particle=16, stiff=0.5, sigma=1.2, n=8, dir=(0.0, 0.0, 1.0), position=1.0 - float(pos[16, 2]),
             only_repulsive=True),
        dict(type="generic_central_force", particle=17, F0=0.7, inner_cut_off=0.5, center=tuple(com + [3.0, 0.0, 0.0])),
        dict(type="repulsion_plane_moving", particle=18, ref_particle=3, stiff=1.7, dir=tuple(u)),
        dict(type="repulsion_plane_moving", particle=18, ref_particle=4, stiff=1.7, dir=tuple(u)),
        dict(type="LJ_cone", particle=19, stiff=1.0, sigma=1.0, n=6, alpha=1.0, dir=(0.0, 0.0, 1.0),
             pos0=tuple(pos[19] - [0.2, 0.1, 1.8])),
        dict(type="twist", particle=6, stiff=1.3, rate=1e-3, base=0.5, axis=(0.0, 0.6, 0.8),
             pos0=tuple(pos[6] + [1.0, 0.5, -0.3]), center=tuple(com), mask=(1.0, 1.0, 0.5)),
        dict(type="ellipsoid", particle=8, stiff=0.6, r_2=(0.4, 0.5, 0.3), center=tuple(com)),
        dict(type="ellipsoid", particle=10, stiff=0.6, r_2=(30.0, 30.0, 30.0), center=tuple(com)),
        dict(type="com", com_list=[20, 22], ref_list=[0, 1, 2, 3], stiff=0.8, r0=1.0, rate=1e-3),
        dict(type="yukawa_sphere", particle=12, radius=float(np.linalg.norm(pos[12] - com)) + 0.8, WCA_epsilon=0.3,
             WCA_sigma=1.0, debye_length=0.5, debye_A=2.0, center=tuple(com)),
        dict(type="repulsive_sphere_moving", particle=23, stiff=0.5, rate=1e-4, origin=tuple(com + [3.0, 0.0, 0.0]),
             target=tuple(com), steps=4000,
             r0=float(np.linalg.norm(pos[23] - (com + [2.25, 0.0, 0.0]))) - 0.6 - 0.1),
    ]


def ext_force_file(forces):
    vec = lambda v: ", ".join(repr(float(x)) for x in v)
    out = []
    for d in forces:
        kv = {"type": d["type"], "particle": d.get("particle")}
        t = d["type"]
        if t == "string":
            kv.update(F0=d["F0"], rate=d["rate"], dir=vec(d["dir"]))
            if d.get("dir_as_centre"):
                kv["dir_as_centre"] = "true"
        elif t == "mutual_trap":
            kv.update(ref_particle=d["ref_particle"], stiff=d["stiff"], r0=d["r0"], rate=d.get("rate", 0.0),
                      stiff_rate=d.get("stiff_rate", 0.0))
            if d.get("PBC"):
                kv["PBC"] = "true"
        elif t == "trap":
            kv.update(stiff=d["stiff"], rate=d["rate"], pos0=vec(d["pos0"]), dir=vec(d["dir"]))
        elif t == "lowdim_trap":
            kv.update(stiff=d["stiff"], rate=d["rate"], pos0=vec(d["pos0"]), dir=vec(d["dir"]),
                      visibility=", ".join(str(int(bool(v))) for v in d["visibility"]))
        elif t == "repulsion_plane":
            kv.update(stiff=d["stiff"], position=d["position"], end_position=d["r0"], v=d["rate"], dir=vec(d["dir"]))
        elif t == "attraction_plane":
            kv.update(stiff=d["stiff"], position=d["position"], dir=vec(d["dir"]))
        elif t == "sphere":
            kv.update(stiff=d["stiff"], r0=d["r0"], rate=d.get("rate", 0.0), center=vec(d["center"]))
            if "r_ext" in d:
                kv["r_ext"] = d["r_ext"]
        elif t == "sphere_smooth":
            # the reference reads the smoothing length and alpha from the key r_ext as well
            # (src/Forces/RepulsiveSphereSmooth.cpp:27-29): the fixture keeps the three equal
            assert d["smooth"] == d["alpha"] == d["r_ext"]
            kv.update(stiff=d["stiff"], r0=d["r0"], r_ext=d["r_ext"], center=vec(d["center"]))
        elif t == "LJ_wall":
            kv.update(stiff=d["stiff"], sigma=d["sigma"], n=d["n"], position=d["position"], dir=vec(d["dir"]))
            if d.get("only_repulsive"):
                kv["only_repulsive"] = "true"
        elif t == "generic_central_force":
            kv.update(force_type="gravity", F0=d["F0"], inner_cut_off=d.get("inner_cut_off", 0.0),
                      outer_cut_off=d.get("outer_cut_off", 0.0), center=vec(d["center"]))
        elif t == "repulsion_plane_moving":
            kv.update(ref_particle=d["ref_particle"], stiff=d["stiff"], dir=vec(d["dir"]))
        elif t == "LJ_cone":
            kv.update(stiff=d["stiff"], sigma=d["sigma"], n=d["n"], alpha=d["alpha"], dir=vec(d["dir"]),
                      pos0=vec(d["pos0"]))
        elif t == "twist":
            kv.update(stiff=d["stiff"], rate=d["rate"], base=d["base"], axis=vec(d["axis"]), pos0=vec(d["pos0"]),
                      center=vec(d["center"]), mask=vec(d["mask"]))
        elif t == "ellipsoid":
            kv.update(stiff=d["stiff"], r_2=vec(d["r_2"]), center=vec(d["center"]))
            if "r_1" in d:
                kv["r_1"] = vec(d["r_1"])
        elif t == "com":
            del kv["particle"]
            kv.update(com_list=",".join(str(i) for i in d["com_list"]), ref_list=",".join(str(i) for i in d["ref_list"]),
                      stiff=d["stiff"], r0=d["r0"], rate=d["rate"])
        elif t == "yukawa_sphere":
            # (the reference reads the key WCA_n into the WCA sigma, YukawaSphere.cpp init: left out)
            kv.update(radius=d["radius"], WCA_epsilon=d["WCA_epsilon"], WCA_sigma=d["WCA_sigma"],
                      debye_length=d["debye_length"], debye_A=d["debye_A"],
                      center=",".join(repr(float(x)) for x in d["center"]))  # its parser takes no spaces
        elif t == "repulsive_sphere_moving":
            kv.update(stiff=d["stiff"], r0=d["r0"], rate=d["rate"], origin=vec(d["origin"]), target=vec(d["target"]),
                      steps=d["steps"])
        out.append("{\n" + "".join(f"{k} = {v}\n" for k, v in kv.items()) + "}\n")
    return "".join(out)


def run_ext_case(name, s, settings, step):
    """the external forces the reference adds at MD step `step` (the configuration's time, kept
    by restart_step_counter = 0): the reference's forces with and without them"""
    import json
    forces = ext_force_set(s.N, float(s.box), s.pos)
    dumps = {}
    with tempfile.TemporaryDirectory() as tmp:
        s.write(os.path.join(tmp, "init.top"), os.path.join(tmp, "init.dat"))
        conf = open(os.path.join(tmp, "init.dat")).read().split("\n", 1)[1]
        open(os.path.join(tmp, "init.dat"), "w").write(f"t = {step}\n" + conf)
        open(os.path.join(tmp, "forces.txt"), "w").write(ext_force_file(forces))
        for tag, ext in (("no", "external_forces = 0\n"),
                         ("ext", "external_forces = 1\nexternal_forces_file = forces.txt\n")):
            text = BASE_INPUT.format(steps=0, dt=0.003, T=settings["T_str"], salt=settings["salt"])
            text = text.replace("restart_step_counter = 1\n", "restart_step_counter = 0\n")
            text = text.replace("external_forces = 0\n", ext)
            open(os.path.join(tmp, "input"), "w").write(text)
            out = os.path.join(tmp, f"dump_{tag}.txt")
            subprocess.run([DUMP, "input", out], cwd=tmp, check=True, stdout=subprocess.DEVNULL,
                           stderr=subprocess.DEVNULL)
            dumps[tag] = parse_dump(out)
    d0, d1 = dumps["no"], dumps["ext"]
    assert d1.get("step") == step, d1.get("step")
    st = d1["state"]
    np.savez_compressed(os.path.join(HERE, name + ".npz"), box=d1["box"][0], step=step, pos=st[:, 0:3],
                        F_ext=d1["forces"][:, 0:3] - d0["forces"][:, 0:3], T_ext=d1["forces"][:, 3:6] - d0["forces"][:, 3:6],
                        forces=json.dumps(forces))
    print(f"{name}: step {step}, max |F_ext| {np.abs(d1['forces'][:, 0:3] - d0['forces'][:, 0:3]).max():.3f}")


def write_system(tmp, s):
    tp, cp = os.path.join(tmp, "s.top"), os.path.join(tmp, "s.dat")
    s.write(tp, cp)
    return tp, cp


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("OXDNA_REFERENCE"),
                    help="oxDNA reference checkout (default: $OXDNA_REFERENCE)")
    ap.add_argument("--only", default=None, help="regenerate this fixture only (ext_forces)")
    args = ap.parse_args()
    if not args.ref:
        ap.error("name the oxDNA reference checkout with --ref or OXDNA_REFERENCE")
    if args.only == "ext_forces":
        if not os.path.exists(DUMP):
            subprocess.run(["make", "-C", os.path.join(REPO, "oracle", "ref"), "-j8", f"REF={args.ref}"], check=True)
        run_ext_case("ext_forces", G.system_for_config(0, seed=1), dict(T_str="300K", salt="0.5"), 1000)
        return
    if not os.path.exists(DUMP):
        subprocess.run(["make", "-C", os.path.join(REPO, "oracle", "ref"), "-j8", f"REF={args.ref}"], check=True)
    ff = os.path.join(args.ref, "test", "DNA", "FORCE_FIELD")

    # 1-2: the reference's own DNA2 force-field test system (16 nt, 3 strands)
    base = dict(T_str="20C", salt="1.0")
    run_case("ff16_avg", os.path.join(ff, "init.top"), os.path.join(ff, "init.dat"), base)
    seq = oxio.read_seq_dep_file(os.path.join(args.ref, "oxDNA2_sequence_dependent_parameters.txt"))
    seq_file = os.path.join(args.ref, "oxDNA2_sequence_dependent_parameters.txt")
    run_case("ff16_seqdep", os.path.join(ff, "init.top"), os.path.join(ff, "init.dat"), dict(base, average=0, seq=seq),
             extra=f"use_average_seq = false\nseq_dep_file = {seq_file}\n")
    # golden split energies the reference's regression test checks (mesh DNA2, 6 decimals)
    gold = {k: np.loadtxt(os.path.join(ff, k, "reference.dat")) for k in ("AVG_SEQ", "SEQ_DEP")}
    np.savez_compressed(os.path.join(HERE, "ff16_reference_dat.npz"), avg_seq=gold["AVG_SEQ"], seq_dep=gold["SEQ_DEP"])

    rng = np.random.default_rng(20240601)
    with tempfile.TemporaryDirectory() as tmp:
        T300 = dict(T_str="300K", salt="0.5")
        # 3: workload-0 system, a 12-bp duplex in a cube of side 20
        s = G.system_for_config(0, seed=1)
        run_case("duplex24", *write_system(tmp, s), T300)

        # 4: a dense mixture exercising every non-bonded term (duplexes, hairpins, coils)
        mols = [G.duplex(G.random_sequence(rng, int(rng.integers(8, 16)))) for _ in range(5)]
        mols += [G.hairpin(G.random_sequence(rng, 7), int(rng.integers(4, 9)), rng) for _ in range(3)]
        mols += [G.random_walk_strand(24, rng) for _ in range(3)]
        s = G.assemble(G.place(mols, 16.0, rng), 16.0, G.kelvin(300), rng)
        # thermal jiggle so that angular terms sample away from their ideal values
        s.pos = s.pos + rng.normal(scale=0.01, size=s.pos.shape)
        s.a1 = s.a1 + rng.normal(scale=0.02, size=s.a1.shape)
        s.a3 = s.a3 + rng.normal(scale=0.02, size=s.a3.shape)
        run_case("mixed", *write_system(tmp, s), T300)
        # the same molecules packed with close contacts: excluded-volume forces up to ~1e5
        s2 = G.assemble(G.place(mols, 16.0, rng, min_dist=0.3), 16.0, G.kelvin(300), rng)
        run_case("contact", *write_system(tmp, s2), T300)

        # 5: different salt, temperature and Debye-Hueckel settings, full charges at the ends
        run_case("dh_variants", *write_system(tmp, s), dict(T_str="330K", salt="0.2", half_charged_ends=0,
                                                            dh_lambda=0.35, dh_strength=0.06),
                 extra="dh_half_charged_ends = false\ndh_lambda = 0.35\ndh_strength = 0.06\n")

        # 6: max_backbone_force with stretched and compressed bonds
        m = G.random_walk_strand(40, rng)
        s = G.assemble(G.place([m], 30.0, rng), 30.0, G.kelvin(300), rng)
        s.pos = s.pos * 1.0 + rng.normal(scale=0.15, size=s.pos.shape)
        run_case("mbf", *write_system(tmp, s), dict(T300, mbf_fmax=5.0, mbf_finf=0.04),
                 extra="max_backbone_force = 5.0\nmax_backbone_force_far = 0.04\n")

        # 7: custom pairing codes >= 300 with an hb_multiplier
        s = G.system_for_config(0, seed=2)
        bt = s.top.btype.copy()
        n = bt.size // 2
        for i in range(n):
            j = bt.size - 1 - i
            if i % 2 == 0:
                bt[i] = 300 + bt[i]
                bt[j] = 3 - bt[i]
        s.top = oxio.Topology(s.top.n3, s.top.n5, bt, np.array([oxio.type_from_btype(int(b)) for b in bt], np.int32),
                              s.top.strand, s.top.n_strands)
        run_case("hbmult", *write_system(tmp, s), dict(T300, hb_multiplier=3.5), extra="hb_multiplier = 3.5\n")

        # 8: integrator pin, 200 NVE steps of a thermal 12-bp duplex
        s = G.system_for_config(0, seed=3)
        run_case("md_nve", *write_system(tmp, s), T300, steps=200, dt=0.003)

    # 9: the external forces of six types at MD step 1000 on the workload-0 duplex
    run_ext_case("ext_forces", G.system_for_config(0, seed=1), dict(T_str="300K", salt="0.5"), 1000)


if __name__ == "__main__":
    main()
