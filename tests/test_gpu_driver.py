"""The caller path end to end on the GPU: a PhysiCell_settings.xml file and an
agents file go through the settings reader, the microenvironment builder, the
solver registry and the gb300 solver plugin (physicore_gb300/examples/diffuse.cpp),
and the VTK images it writes are compared with the oracle stepped on the same
problem: 1e-12 relative per substrate for the FP64 solver, 1e-5 for FP32."""
import os
import subprocess

import numpy as np
import pytest

from test_gpu_golden import rel_err
from vti import read_pvd, read_vti

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
BUILD = os.path.join(ROOT, "tests", "_build")
FACES = ("xmin", "xmax", "ymin", "ymax", "zmin", "zmax")


@pytest.fixture(scope="module")
def diffuse_exe(pcg):
    from physicore_gb300 import _build
    host_lib = _build.build_host()
    os.makedirs(BUILD, exist_ok=True)
    exe = os.path.join(BUILD, "diffuse")
    pkg = os.path.dirname(host_lib)
    subprocess.run([_build.cxx(), "-std=c++20", "-O2", "-Wall", "-Wextra",
                    os.path.join(ROOT, "physicore_gb300", "examples", "diffuse.cpp"),
                    "-I", os.path.join(ROOT, "include"), "-L", pkg, "-lphysicore_gb300_host", "-lphysicore_gb300",
                    f"-Wl,-rpath,{pkg}", "-o", exe], check=True)
    return exe


def _problem(seed, dims):
    """A random settings file's content as the oracle's problem, with its XML."""
    rng = np.random.default_rng(seed)
    S = 3
    voxel = [int(v) for v in rng.choice([8, 10, 12], 3)]
    n = [int(v) for v in rng.integers(9, 26, 3)]
    lo = [int(v) for v in rng.integers(-300, 100, 3)]
    if dims == 2:
        n[2] = 1
    hi = [lo[a] + n[a] * voxel[a] for a in range(3)]
    dt = float(rng.choice([0.01, 0.02, 0.05]))
    # plain floats: repr of a numpy scalar is not a number to strtod
    D = [float(v) for v in 10.0 ** rng.uniform(1, 4.5, S)]
    decay = [float(v) for v in 10.0 ** rng.uniform(-3, 0, S)]
    initial = [float(v) for v in rng.uniform(0, 10, S)]
    # substrate 0: legacy condition then per-face overrides; others: per-face only
    faces = np.zeros((S, 6), bool)
    values = np.zeros((S, 6))
    var_xml = []
    for s in range(S):
        lines = []
        if s == 0:
            v = float(rng.uniform(0, 20))
            faces[s, :] = True
            values[s, :] = v
            lines.append(f'<Dirichlet_boundary_condition enabled="true">{v!r}</Dirichlet_boundary_condition>')
        opts = []
        for f in range(6):
            if rng.random() < 0.5:
                on = bool(rng.random() < 0.6)
                v = float(rng.uniform(0, 20))
                faces[s, f], values[s, f] = on, v
                opts.append(f'<boundary_value ID="{FACES[f]}" enabled="{str(on).lower()}">{v!r}</boundary_value>')
        if opts:
            lines.append("<Dirichlet_options>" + "".join(opts) + "</Dirichlet_options>")
        var_xml.append(f'''
        <variable name="sub{s}" units="mM" ID="{s}">
            <physical_parameter_set>
                <diffusion_coefficient>{D[s]!r}</diffusion_coefficient>
                <decay_rate>{decay[s]!r}</decay_rate>
            </physical_parameter_set>
            <initial_condition>{initial[s]!r}</initial_condition>
            {"".join(lines)}
        </variable>''')
    xml = f'''<?xml version="1.0"?>
<PhysiCell_settings>
    <domain>
        <x_min>{lo[0]}</x_min><x_max>{hi[0]}</x_max>
        <y_min>{lo[1]}</y_min><y_max>{hi[1]}</y_max>
        <z_min>{lo[2]}</z_min><z_max>{hi[2]}</z_max>
        <dx>{voxel[0]}</dx><dy>{voxel[1]}</dy><dz>{voxel[2]}</dz>
        <use_2D>{"true" if dims == 2 else "false"}</use_2D>
    </domain>
    <overall>
        <max_time>1.0</max_time><time_units>min</time_units><space_units>micron</space_units>
        <dt_diffusion>{dt!r}</dt_diffusion><dt_mechanics>0.1</dt_mechanics><dt_phenotype>6</dt_phenotype>
    </overall>
    <microenvironment_setup>{"".join(var_xml)}
        <options><track_internalized_substrates_in_each_agent>true</track_internalized_substrates_in_each_agent></options>
    </microenvironment_setup>
</PhysiCell_settings>
'''
    A = int(rng.integers(50, 400))
    pos = np.stack([rng.uniform(lo[a], hi[a], A) for a in range(3)], axis=1)
    pos = np.minimum(pos, np.nextafter(np.asarray(hi, float), -np.inf))
    # a few agents share voxels
    pos[: A // 4] = pos[A // 4: 2 * (A // 4)]
    agents = dict(positions=np.ascontiguousarray(pos[:, :dims]), volumes=rng.uniform(1000, 3000, A),
                  secretion=rng.uniform(0, 5, (A, S)), saturation=rng.uniform(0, 20, (A, S)),
                  uptake=rng.uniform(0, 2, (A, S)), net_export=rng.uniform(0, 0.5, (A, S)),
                  is_active=np.ones(A, np.uint8), fraction_released=np.zeros((A, S)))
    rows = [f"{A} {S}"]
    for i in range(A):
        vals = list(pos[i]) + [agents["volumes"][i]]
        for k in ("secretion", "saturation", "uptake", "net_export"):
            vals += list(agents[k][i])
        rows.append(" ".join(repr(float(v)) for v in vals))
    boundary = []
    for a in range(dims):
        for side in range(2):
            f = 2 * a + side
            if faces[:, f].any():
                boundary.append((a, side, list(values[:, f]), [int(c) for c in faces[:, f]]))
    p = dict(name=f"driver_{seed}", dims=dims, bbmin=tuple(lo), bbmax=tuple(hi), voxel=tuple(voxel), dt=dt, D=D,
             decay=decay, initial=initial, boundary=boundary, agents=agents, compute_internalized=True, field=None)
    return p, xml, "\n".join(rows) + "\n"


def _run(exe, workdir, xml, agents_txt, steps, solver, extra=()):
    settings = os.path.join(workdir, "settings.xml")
    open(settings, "w").write(xml)
    agents = os.path.join(workdir, "agents.txt")
    open(agents, "w").write(agents_txt)
    out = os.path.join(workdir, "out")
    r = subprocess.run([exe, settings, "--output", out, "--agents", agents, "--steps", str(steps),
                        "--interval", "1e9", "--solver", solver, *extra],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    entries = read_pvd(os.path.join(out, "microenvironment.pvd"))
    return r.stdout, [read_vti(os.path.join(out, f)) for _, f in entries], entries


@pytest.mark.parametrize("seed,dims,solver", [(0, 3, "gb300_solver"), (1, 2, "gb300_solver"),
                                              (2, 3, "gb300_solver_fp32"), (3, 2, "gb300_solver_fp32")])
def test_driver_matches_oracle(diffuse_exe, oracle_mod, tmp_path, seed, dims, solver):
    from physicore_gb300 import workloads as W
    p, xml, agents_txt = _problem(seed, dims)
    steps = 7
    _, images, entries = _run(diffuse_exe, str(tmp_path), xml, agents_txt, steps, solver)
    assert len(images) == 2 and entries[1][0] == pytest.approx(steps * p["dt"], rel=1e-6)
    o = W.apply(oracle_mod.OracleSolver(threads=2), p)
    ref0 = o.get_field()
    for _ in range(steps):  # the driver's loop: one solve call per step
        o.solve(1)
    ref = o.get_field()
    rtol = 1e-12 if solver == "gb300_solver" else 1e-5
    for k, (img, want) in enumerate(((images[0], ref0), (images[1], ref))):
        assert list(img["arrays"]) == [f"sub{s}" for s in range(3)]
        got = np.stack([img["arrays"][f"sub{s}"] for s in range(3)], axis=-1)
        err = rel_err(got, want)
        assert err <= rtol, f"image {k}: max-rel {err:.3e} > {rtol}"


def test_driver_transfer_every_step_same_field(diffuse_exe, tmp_path):
    """The reference's loop (field to and from the device around every step) and
    the resident loop write the same images, to the FP32 tolerance: the round trip
    through the FP64 host mirror is exact, but sums over agents sharing a voxel
    are atomics in any order, so two runs need not be bit-equal."""
    p, xml, agents_txt = _problem(5, 3)
    a = tmp_path / "resident"
    b = tmp_path / "transfer"
    a.mkdir()
    b.mkdir()
    _, ia, _ = _run(diffuse_exe, str(a), xml, agents_txt, 6, "gb300_solver_fp32")
    _, ib, _ = _run(diffuse_exe, str(b), xml, agents_txt, 6, "gb300_solver_fp32", ("--transfer-every-step",))
    for name in ia[-1]["arrays"]:
        assert rel_err(ia[-1]["arrays"][name], ib[-1]["arrays"][name]) <= 1e-5, name


def test_example_settings_run(diffuse_exe, tmp_path):
    """The example settings file with its built-in agent clusters: outputs at the
    requested interval and a summary line."""
    settings = os.path.join(ROOT, "physicore_gb300", "examples", "settings.xml")
    out = str(tmp_path / "out")
    r = subprocess.run([diffuse_exe, settings, "--output", out, "--steps", "50", "--interval", "0.5"],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "[diffuse] done: steps=50" in r.stdout
    entries = read_pvd(os.path.join(out, "microenvironment.pvd"))
    assert [round(t, 6) for t, _ in entries] == [0.0, 0.5, 1.0]
    img = read_vti(os.path.join(out, entries[-1][1]))
    assert list(img["arrays"]) == ["oxygen", "glucose", "lactate"]
    assert img["extent"] == [-60, 60, -60, 60, 0, 0]
    ox = img["arrays"]["oxygen"][0]
    # Dirichlet faces of the example: x-min 64, x-max 30 (y-min 52 set after x)
    assert np.all(ox[1:-1, 0] == 64.0) and np.all(ox[1:-1, -1] == 30.0) and np.all(ox[0, :] == 52.0)
    lac = img["arrays"]["lactate"][0]
    assert np.all(np.isfinite(lac)) and lac.min() >= 0.0 and lac.max() == 0.0  # no agent secretes lactate
