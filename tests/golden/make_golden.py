"""Regenerate the golden fixtures from the reference's own CPU solver.

Run in a container that has the reference sources (the GPU hosts do not):

    oracle/build_ref.sh && python tests/golden/make_golden.py

For every case below it runs oracle/_ref/ref_harness (the reference's
LBMSolver, built from source) for the listed step counts and stores the grid
tables, the JSON ``solver`` block and the resulting populations, variables and
residual in tests/golden/<case>_<steps>.npz (and, for VTP_CASES, the
reference's own VTK output file).  The case configs are either the
project's own JSON files in tests/golden/cases/ (written in the reference's
config schema) or the reference's own test configs, read where they lie.
"""
from __future__ import annotations

import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
HARNESS = os.path.join(ROOT, "oracle", "_ref", "ref_harness")
# the reference checkout, as the build recipe of the harness resolves it
REF = subprocess.run([os.path.join(ROOT, "oracle", "build_ref.sh"), "--root"], capture_output=True, text=True,
                     check=True).stdout.strip()

# (fixture name, config path, step counts)
CASES = [
    ("couette", ("ref", "test/couette/couette.json"), [1, 50, 1000]),
    ("couette_bnd", ("ref", "test/couette/couette_bnd.json"), [1, 50]),
    ("couette_bnd_bbDirichlet", ("ref", "test/couette/couette_bnd_bbDirichlet.json"), [50]),
    ("couette_bnd_eq", ("ref", "test/couette/couette_bnd_eq.json"), [50, 1000]),
    ("couette_bnd_eq2", ("ref", "test/couette/couette_bnd_eq2.json"), [50]),
    ("couette_bnd_NEEM", ("ref", "test/couette/couette_bnd_NEEM.json"), [50, 1000]),
    ("couette_bnd_NEBB", ("ref", "test/couette/couette_bnd_NEBB.json"), [50, 1000]),
    ("poiseuille", ("ref", "test/poiseuille/poiseuille.json"), [1, 50, 1000]),
    ("poiseuille_bnd", ("ref", "test/poiseuille/poiseuille_bnd.json"), [50]),
    ("poiseuille_bnd_eq", ("ref", "test/poiseuille/poiseuille_bnd_eq.json"), [50]),
    ("poiseuille_bnd_NEEM", ("ref", "test/poiseuille/poiseuille_bnd_NEEM.json"), [50]),
    ("poiseuille_bnd_NEBB", ("ref", "test/poiseuille/poiseuille_bnd_NEBB.json"), [50]),
    ("poiseuille_bnd_pressure", ("ref", "test/poiseuille/poiseuille_bnd_pressure.json"), [50, 1000]),
    ("poiseuille_bnd_pressure_neem2", ("ref", "test/poiseuille/poiseuille_bnd_pressure_neem2.json"), [50]),
    ("poisson1D_reaction", ("ref", "test/poisson/poisson1D_reaction.json"), [50, 1000]),
    ("poisson1d_dh_small", ("own", "poisson1d_dh_small.json"), [1, 100]),
    ("poisson2d_d2q5_small", ("own", "poisson2d_d2q5_small.json"), [1, 100]),
    ("poisson2d_d2q9_reaction_small", ("own", "poisson2d_d2q9_reaction_small.json"), [100]),
    ("poisson2d_helmholtz_small", ("own", "poisson2d_helmholtz_small.json"), [100, 1000]),
    ("cavity_small", ("own", "cavity_small.json"), [1, 100, 1000]),
    ("channel_mixed_small", ("own", "channel_mixed_small.json"), [1, 100]),
    # the reference's remaining Poisson tests and its backward-facing steps
    # (bodies made of several boxes), at coarser levels
    ("poisson1D_l8", ("ref", "test/poisson/poisson1D.json", {"partitionLevel": 8, "uniformLevel": 8, "maxRfnmtLvl": 8}), [50]),
    ("poisson2D_l5", ("ref", "test/poisson/poisson2D.json", {"partitionLevel": 5, "uniformLevel": 5, "maxRfnmtLvl": 5}), [50]),
    ("poisson2D_reaction_l5", ("ref", "test/poisson/poisson2D_reaction.json",
                               {"partitionLevel": 5, "uniformLevel": 5, "maxRfnmtLvl": 5}), [50]),
    ("poissonD2Q9_l5", ("ref", "test/poisson/poissonD2Q9.json", {"partitionLevel": 5, "uniformLevel": 5, "maxRfnmtLvl": 5}), [50]),
    ("step_ns_l5", ("ref", "test/step/step_ns.json", {"partitionLevel": 5, "uniformLevel": 5, "maxRfnmtLvl": 5}), [40, 1000]),
    ("step_poisson_l5", ("ref", "test/step/step_poisson.json", {"partitionLevel": 5, "uniformLevel": 5, "maxRfnmtLvl": 5}), [40]),
    # the reference's 2D flow around an obstacle (box minus a circle, pressure
    # inlet / outlet, bounce-back walls) at level 5 instead of 8
    ("sphere_ns_l5", ("ref", "test/sphere/sphere_ns.json", {"partitionLevel": 5, "uniformLevel": 5, "maxRfnmtLvl": 5}),
     [1, 60, 1000]),
    # multi-level grids: the solver loads every level of the generator's array
    # and steps each as a lattice of its own (src/lbm/solver.cpp:525)
    ("poiseuille_p3u5", ("ref", "test/poiseuille/poiseuille.json", {"partitionLevel": 3, "uniformLevel": 5, "maxRfnmtLvl": 5}),
     [20, 1000]),
    ("cavity_p2u3m5", ("own", "cavity_small.json", {"partitionLevel": 2, "uniformLevel": 3, "maxRfnmtLvl": 5}), [100]),
    ("cavity_obstacle_p2u3m6", ("own", "cavity_obstacle_small.json", {"partitionLevel": 2, "uniformLevel": 3, "maxRfnmtLvl": 6}),
     [100]),
    ("poisson2d_helmholtz_p2u3m5", ("own", "poisson2d_helmholtz_small.json",
                                    {"partitionLevel": 2, "uniformLevel": 3, "maxRfnmtLvl": 5}), [100]),
]


def config_path(src):
    kind, rel = src[0], src[1]
    return os.path.join(REF, rel) if kind == "ref" else os.path.join(HERE, "cases", rel)


def load_config(src):
    """The case's JSON config; a third element of ``src`` holds top-level keys
    that replace the file's (a reference test case at a coarser level)."""
    with open(config_path(src)) as fh:
        cfg = json.load(fh)
    if len(src) > 2:
        cfg.update(src[2])
    return cfg


def run_case(name, src, steps):
    cfg = load_config(src)
    with tempfile.TemporaryDirectory() as tmp:
        # the harness writes logs into its working directory
        local_cfg = os.path.join(tmp, "case.json")
        with open(local_cfg, "w") as fh:
            json.dump(cfg, fh)
        out = os.path.join(tmp, "out")
        os.makedirs(out)
        subprocess.run([HARNESS, local_cfg, str(steps), out], cwd=tmp, check=True,
                       stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
        with open(os.path.join(out, "meta.json")) as fh:
            meta = json.load(fh)
        arrays = {}
        for key, dtype in (("centers", np.float64), ("nghbr", np.int64), ("fold0", np.float64), ("fold", np.float64),
                           ("vars", np.float64), ("varsold", np.float64), ("residual", np.float64)):
            arrays[key] = np.fromfile(os.path.join(out, f"{key}.{ 'i64' if dtype is np.int64 else 'f64'}"), dtype=dtype)
    np.savez_compressed(os.path.join(HERE, f"{name}_{steps}.npz"), meta=json.dumps(meta), solver=json.dumps(cfg["solver"]),
                        **arrays)
    print(f"{name}_{steps}: {meta['cells']} cells")


# cases whose final state the reference also writes through its own VTK
# output (LBMSolver::output, binary PolyData): tests/golden/<case>_<steps>_ref.vtp
VTP_CASES = [("cavity_small", 100), ("poisson2d_helmholtz_small", 100), ("cavity_p2u3m5", 100)]


def run_vtp(name, steps):
    src = next(s for n, s, _ in CASES if n == name)
    cfg = load_config(src)
    with tempfile.TemporaryDirectory() as tmp:
        local_cfg = os.path.join(tmp, "case.json")
        with open(local_cfg, "w") as fh:
            json.dump(cfg, fh)
        out = os.path.join(tmp, "out")
        os.makedirs(out)
        subprocess.run([HARNESS, local_cfg, str(steps), out, "--vtp"], cwd=tmp, check=True, stdout=subprocess.DEVNULL,
                       stderr=subprocess.DEVNULL)
        files = [f for f in os.listdir(out) if f.startswith("solution") and f.endswith(".vtp")]
        if len(files) != 1:
            sys.exit(f"{name}: expected one .vtp file, found {files}")
        with open(os.path.join(out, files[0]), "rb") as fh:
            data = fh.read()
    with open(os.path.join(HERE, f"{name}_{steps}_ref.vtp"), "wb") as fh:
        fh.write(data)
    print(f"{name}_{steps}_ref.vtp: {len(data)} bytes")


# line probes (the reference's "postprocessing" line objects, executed at the
# end of the run, src/postprocess/postprocessing.h:87-119): the reference's own
# line.csv after <steps> steps -> tests/golden/<case>_<steps>_line_<tag>.csv.
# Lines run through cell centres along an axis or with a positive slope: there
# the reference's sort comparator is a strict weak order, so its cell order is
# defined.
LINE_CASES = [
    ("cavity_small", 100, "x0p53", [0.53125, 0.0], [0.53125, 1.0]),
    ("cavity_small", 100, "diag", [0.0, 0.0], [1.0, 1.0]),
    ("poisson2d_helmholtz_small", 100, "y0p41", [0.0, 0.40625], [1.0, 0.40625]),
    ("channel_mixed_small", 100, "x1p06", [1.0625, 0.0], [1.0625, 1.0]),
]


def run_line(name, steps, tag, a, b):
    src = next(s for n, s, _ in CASES if n == name)
    cfg = load_config(src)
    cfg["solver"]["postprocessing"] = {"line1": {"type": "line", "execute": "atEnd", "A": a, "B": b}}
    with tempfile.TemporaryDirectory() as tmp:
        local_cfg = os.path.join(tmp, "case.json")
        with open(local_cfg, "w") as fh:
            json.dump(cfg, fh)
        out = os.path.join(tmp, "out")
        os.makedirs(out)
        subprocess.run([HARNESS, local_cfg, str(steps), out], cwd=tmp, check=True, stdout=subprocess.DEVNULL,
                       stderr=subprocess.DEVNULL)
        with open(os.path.join(tmp, "line.csv"), "rb") as fh:
            data = fh.read()
    dst = os.path.join(HERE, f"{name}_{steps}_line_{tag}.csv")
    with open(dst, "wb") as fh:
        fh.write(data)
    print(f"{os.path.basename(dst)}: {data.count(b'\n') - 1} points")


# the grid part of every case's config (grid generator keys, geometry and the
# solver's boundary block): tests/golden/grid_configs.json, the input of the
# grid-table tests (the reference's own test configs are not read at test time)
GRID_KEYS = ("dim", "partitionLevel", "uniformLevel", "maxRfnmtLvl", "maxNoCells", "boundingBox", "alignNodesWithSurface", "alignDir",
             "geometry")


def write_grid_configs():
    out = {}
    for name, src, _ in CASES:
        cfg = load_config(src)
        g = {k: cfg[k] for k in GRID_KEYS if k in cfg}
        g["solver"] = {"boundary": cfg["solver"]["boundary"]}
        out[name] = g
    with open(os.path.join(HERE, "grid_configs.json"), "w") as fh:
        json.dump(out, fh, indent=1, sort_keys=True)
        fh.write("\n")
    print(f"grid_configs.json: {len(out)} cases")


# particle solver (src/lpt): the reference's own LPTSolver through
# oracle/_ref/ref_lpt_harness -> tests/golden/lpt_<case>_<steps>.npz with the
# particle state before and after (the solver's m_vars layout), the start
# locations and the constants.  The reference's freefall tests, shortened, and
# the same case with the other force models (ambient velocity set, so that the
# drag acts on a moving fluid) and integrators.
LPT_HARNESS = os.path.join(ROOT, "oracle", "_ref", "ref_lpt_harness")
LPT_MODELS = [("constDensityRatioGrav", "ForwardEuler", 2), ("constDensityRatioGravStokesDrag", "ImplicitEuler", 3),
              ("constDensityRatioGravNlinDrag", "ImplicitEuler", 2), ("constDensityRatioGravBuo", "ForwardEuler", 3),
              ("constDensityRatioGravBuoStokesDrag", "ForwardEuler", 2), ("constDensityRatioGravBuoNlinDrag", "ForwardEuler", 3),
              ("constDensityaGravBuoStokesDrag", "ImplicitEuler", 2), ("constDensityaGravBuoNlinDrag", "ImplicitEuler", 3)]
LPT_CASES = [(f"lpt_{n}", ("ref", f"test/lpt/{n}.json"), 2000) for n in
             ("falling", "falling_implicit", "falling_nonlinearDrag", "falling_Buoyancy", "falling_noDrag", "falling3d")]


def lpt_model_config(model, integration, dim):
    base = "falling3d.json" if dim == 3 else "falling.json"
    with open(os.path.join(REF, "test", "lpt", base)) as fh:
        cfg = json.load(fh)
    s = cfg["solver"]
    s["model"] = model
    s["integrationMethod"] = integration
    s["v_infty"] = [0.3, -0.2, 0.1][:dim]
    s["rho_infty"] = 1.1
    s["dt"] = 1e-4
    s["randomvol_pos"]["init_rho_p"] = 50.0
    s["randomvol_pos"]["init_velo"] = [0.5, 0.25, -0.1][:dim]
    return cfg


def run_lpt(name, cfg, steps):
    with tempfile.TemporaryDirectory() as tmp:
        local_cfg = os.path.join(tmp, "case.json")
        with open(local_cfg, "w") as fh:
            json.dump(cfg, fh)
        out = os.path.join(tmp, "out")
        os.makedirs(out)
        subprocess.run([LPT_HARNESS, local_cfg, str(steps), out], cwd=tmp, check=True, stdout=subprocess.DEVNULL,
                       stderr=subprocess.DEVNULL)
        with open(os.path.join(out, "meta.json")) as fh:
            meta = json.load(fh)
        arrays = {k: np.fromfile(os.path.join(out, f"{k}.f64"), dtype=np.float64) for k in ("vars0", "vars", "start")}
    np.savez_compressed(os.path.join(HERE, f"{name}_{steps}.npz"), meta=json.dumps(meta), solver=json.dumps(cfg["solver"]), **arrays)
    print(f"{name}_{steps}: {meta['particles']} particles")


def write_lpt():
    for name, src, steps in LPT_CASES:
        run_lpt(name, load_config(src), steps)
    # particle injection (3D): the reference's injection test, 100 steps
    run_lpt("lpt_injection", load_config(("ref", "test/lpt/injection.json")), 100)
    for model, integration, dim in LPT_MODELS:
        run_lpt(f"lpt_{model}_{dim}d", lpt_model_config(model, integration, dim), 2000)


# known answers of the reference's curve index (UnitTest/test_hilbert.cpp):
# every EXPECT_EQ(hilbert::index<N>(point, level), value) with its point ->
# tests/golden/hilbert_kat.json
def write_hilbert_kat():
    import re
    src = open(os.path.join(REF, "UnitTest", "test_hilbert.cpp")).read()
    points, kat = {}, []
    for line in src.splitlines():
        m = re.match(r"\s*VectorD<(\d)>\s+(\w+)\s*=\s*\{([^}]*)\};", line)
        if m:
            points[m.group(2)] = [float(v) for v in m.group(3).split(",")]
            continue
        m = re.match(r"\s*EXPECT_EQ\(hilbert::index<(\d)>\((\w+),\s*(\d+)\),\s*(\d+)\);", line)
        if m:
            kat.append({"ndim": int(m.group(1)), "x": points[m.group(2)], "level": int(m.group(3)), "index": int(m.group(4))})
    with open(os.path.join(HERE, "hilbert_kat.json"), "w") as fh:
        json.dump(kat, fh, indent=0)
        fh.write("\n")
    print(f"hilbert_kat.json: {len(kat)} known answers")


# the reference's analytic test suite (test/run.sh: every LBM case whose config
# carries analyticalSolution): the reference's own run() to convergence, its
# step count and its analytic errors (compareToAnalyticalResult,
# src/lbm/solver.cpp:387-482) at 17 digits -> tests/golden/analytic_suite.json,
# with each case's config (the GPU test builds the grid from it natively)
ANALYTIC_CASES = [(n, ("ref", f"test/couette/{n}.json")) for n in (
    "couette", "couette_bnd", "couette_bnd_bbDirichlet", "couette_bnd_eq", "couette_bnd_eq2", "couette_bnd_NEEM", "couette_bnd_NEBB",
    "couette_bnd_eq_aligned")] + [(n, ("ref", f"test/poiseuille/{n}.json")) for n in (
    "poiseuille", "poiseuille_bnd", "poiseuille_bnd_eq", "poiseuille_bnd_NEBB", "poiseuille_bnd_NEEM", "poiseuille_bnd_pressure_neem2",
    "poiseuille_bnd_pressure")] + [(n, ("ref", f"test/poisson/{n}.json")) for n in (
    "poisson1D", "poisson1D_reaction", "poisson2D_helmholtz")]


def run_analytic(name, src):
    import re
    import time
    cfg = load_config(src)
    with tempfile.TemporaryDirectory() as tmp:
        local_cfg = os.path.join(tmp, "case.json")
        with open(local_cfg, "w") as fh:
            json.dump(cfg, fh)
        out = os.path.join(tmp, "out")
        os.makedirs(out)
        t0 = time.time()
        p = subprocess.run([HARNESS, local_cfg, "0", out, "--run"], cwd=tmp, check=True, capture_output=True, text=True)
        wall = time.time() - t0
    res = json.loads(p.stdout.strip().splitlines()[-1])

    def grab(label):
        m = re.findall(re.escape(label) + r"\s*([-+0-9.eEinfa]+)", p.stderr)
        return float(m[-1]) if m else None

    entry = {"config": cfg, "steps": res["steps"], "diverged": res["diverged"], "converged_to": grab("Reached convergence to:"),
             "max": grab("max. Error:"), "l2": grab("avg. L2:"), "gre": grab("global relative error:")}
    print(f"{name}: {entry['steps']} steps, max {entry['max']}, L2 {entry['l2']}, GRE {entry['gre']} ({wall:.1f} s)", flush=True)
    return entry


def write_analytic(wanted=()):
    path = os.path.join(HERE, "analytic_suite.json")
    suite = {}
    if os.path.exists(path):
        with open(path) as fh:
            suite = json.load(fh)
    for name, src in ANALYTIC_CASES:
        if wanted and name not in wanted and "analytic" not in wanted:
            continue
        suite[name] = run_analytic(name, src)
        with open(path, "w") as fh:
            json.dump(suite, fh, indent=1, sort_keys=True)
            fh.write("\n")


def main(argv):
    if not os.path.exists(HARNESS):
        sys.exit("build the reference first: oracle/build_ref.sh")
    wanted = set(argv[1:])
    if not wanted or "grid_configs" in wanted:
        write_grid_configs()
    if not wanted or "hilbert_kat" in wanted:
        write_hilbert_kat()
    if not wanted or "lpt" in wanted:
        write_lpt()
    if not wanted or "analytic" in wanted or wanted & {n for n, _ in ANALYTIC_CASES}:
        write_analytic(wanted)
    for name, src, steps in CASES:
        if wanted and name not in wanted:
            continue
        for n in steps:
            run_case(name, src, n)
    for name, steps in VTP_CASES:
        if wanted and name not in wanted:
            continue
        run_vtp(name, steps)
    for name, steps, tag, a, b in LINE_CASES:
        if wanted and name not in wanted:
            continue
        run_line(name, steps, tag, a, b)


if __name__ == "__main__":
    main(sys.argv)
