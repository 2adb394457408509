"""End-to-end pyrandaSim on the GPU against the reference goldens and the oracle.

The scripts are the reference's regression scripts (tests/scripts.py); the
product must reproduce the reference's golden scalars within the reference's
tolerance (1e-4 relative) and the oracle's fields to relative L2 <= 1e-12.
"""
import json
import os

import numpy
import pytest

from tests import scripts
from tests.helpers import rel_l2, to_host

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_scalars.json")))["values"]


def _close(v, name, tol=1.0e-4):
    g = GOLD[name]["value"]
    rel = abs(v - g) / abs(g)
    assert rel < tol, (name, v, g, rel)
    return rel


def _ts(ss):
    from pyranda_gb300 import pyrandaTimestep
    ss.addPackage(pyrandaTimestep(ss))


def _bc_ts(ss):
    from pyranda_gb300 import pyrandaBC, pyrandaTimestep
    ss.addPackage(pyrandaBC(ss))
    ss.addPackage(pyrandaTimestep(ss))


def test_unit_test_golden():
    from pyranda_gb300 import pyrandaSim
    err = scripts.unit_test(pyrandaSim, silent=True)
    assert _close(err, "unit-test-3D") < 1e-9


@pytest.mark.parametrize("n", [50, 100, 200, 300, 400])
def test_advection_golden(n):
    from pyranda_gb300 import pyrandaSim
    err = scripts.advection_1d(pyrandaSim, n, silent=True)
    _close(err, "advec-1d-%d" % n)


def test_taylor_green_golden():
    from pyranda_gb300 import pyrandaSim
    enst = scripts.taylor_green(pyrandaSim, 32, 0.1, _ts, silent=True)
    assert _close(enst, "taylorgreen") < 1e-9


def test_shu_osher_golden():
    """tests/cases/testShuOsher.py shu-osher-CR, with every RK step replayed
    from a CUDA graph (bit-identical to eager, test_graph_replay_matches_eager):
    graph capture with the boundary-condition lines of the EOM."""
    from pyranda_gb300 import pyrandaSim
    cr = scripts.shu_osher(pyrandaSim, _bc_ts, graphs=True, silent=True)
    assert _close(cr, "shu-osher-CR") < 1e-8


def test_taylor_green_fields_match_oracle(oracle):
    """Every TGV field after 3 RK steps agrees with the oracle to 1e-12 (relative L2)."""
    from pyranda_gb300 import pyrandaSim
    ss = scripts.make_tgv(pyrandaSim, 24, _ts, silent=True)
    so = scripts.make_tgv(oracle.OracleSim, 24, lambda s: s.addPackage("Timestep"))
    dt = float(ss.variables["dt"].data) * 0.5
    dto = so.variables["dt"].data * 0.5
    assert abs(dt - dto) <= 1e-14 * dto
    t = to = 0.0
    for _ in range(3):
        t = ss.rk4(t, dt)
        to = so.rk4(to, dto)
        dt = float(ss.variables["dt"].data) * 0.5
        dto = so.variables["dt"].data * 0.5
    for name in ["rho", "rhou", "rhov", "rhow", "Et", "u", "p", "mu", "tauxx", "enst"]:
        a = to_host(ss.variables[name].data)
        b = so.variables[name].data
        assert rel_l2(a, b) <= 1e-12, (name, rel_l2(a, b))
    # beta = gbar(|ring(div)| rho): the TGV dilatation is analytically zero, so
    # div is a sum of O(1) terms cancelling to rounding level and ring() takes
    # its 8th derivative; the bound scales with that cancellation.
    ux, vy, wz, div = (so.variables[k].data for k in ("ux", "vy", "wz", "div"))
    cancel = numpy.abs(ux).max() / max(numpy.abs(div).max(), 1e-300)
    e = rel_l2(to_host(ss.variables["beta"].data), so.variables["beta"].data)
    assert e <= 1e-13 * cancel * 4200.0, (e, cancel)


def test_fp32_path_error_bound():
    """The single-precision sweeps stay within 1e-6 (relative L2) of FP64 over 10 TGV steps."""
    from pyranda_gb300 import pyrandaSim
    s64 = scripts.make_tgv(pyrandaSim, 32, _ts, silent=True)
    s32 = scripts.make_tgv(pyrandaSim, 32, _ts, silent=True, precision="fp32")
    dt = float(s64.variables["dt"].data) * 0.5
    t = 0.0
    for _ in range(10):
        s64.rk4(t, dt)
        t = s32.rk4(t, dt)
    for name in ["rho", "rhou", "rhov", "Et"]:
        e = rel_l2(to_host(s32.variables[name].data), to_host(s64.variables[name].data))
        assert e <= 1e-6, (name, e)


@pytest.mark.parametrize("form", ["fp32-split", "auto"])
def test_fast_sweeps_in_the_eom_stay_close_to_fp64(form):
    """The split-line FP32 sweeps (register-resident along every direction of a
    64^3 grid) and the autotuned path inside whole TGV RK steps, with graphs
    and fused EOM kernels: every sweep epilogue of the step (store, the
    divergence's accumulate, the ring's running max, the filters' FP64
    add-back) runs there.  After 10 steps every conserved field is within
    1e-6 relative L2 of the FP64 run (momentum components against the
    momentum vector's norm, since rhow starts at zero)."""
    from pyranda_gb300 import pyrandaSim
    s64 = scripts.make_tgv(pyrandaSim, 64, _ts, silent=True)
    sf = scripts.make_tgv(pyrandaSim, 64, _ts, silent=True, precision="auto" if form == "auto" else "fp32")
    if form == "fp32-split":
        sf.grid.set_line_split(True)
    sf.use_fusion(True)
    sf.use_graphs(True)
    dt = float(s64.variables["dt"].data) * 0.5
    t = 0.0
    for _ in range(10):
        s64.rk4(t, dt)
        t = sf.rk4(t, dt)
    mom = ["rhou", "rhov", "rhow"]
    mnorm = sum(float(numpy.linalg.norm(to_host(s64.variables[n].data).ravel())) ** 2 for n in mom) ** 0.5
    for name in ["rho", "rhou", "rhov", "rhow", "Et"]:
        a, b = to_host(sf.variables[name].data), to_host(s64.variables[name].data)
        ref = mnorm if name in mom else float(numpy.linalg.norm(b.ravel()))
        e = float(numpy.linalg.norm((a - b).ravel())) / ref
        print(form, name, "%.2e" % e)
        assert e <= 1e-6, (form, name, e)


def test_graph_replay_matches_eager():
    """A CUDA-graph replayed rk4 step gives the eager result bit for bit."""
    from pyranda_gb300 import pyrandaSim
    se = scripts.make_tgv(pyrandaSim, 24, _ts, silent=True)
    sg = scripts.make_tgv(pyrandaSim, 24, _ts, silent=True)
    sg.use_graphs(True)
    dt = se.variables["dt"].data * 0.5
    dtg = sg.variables["dt"].data * 0.5
    t = tg = 0.0
    for _ in range(4):
        t = se.rk4(t, dt)
        tg = sg.rk4(tg, dtg)
        dt = se.variables["dt"].data * 0.5
        dtg = sg.variables["dt"].data * 0.5
    torch.cuda.synchronize()
    for name in ["rho", "rhou", "Et", "u", "mu", "dt"]:
        a, b = se.variables[name].data, sg.variables[name].data
        assert torch.equal(a, b), name


def _fields_match(ss, so, names, tol=1e-12, scale=None):
    """Relative L2 per field; a field named in `scale` is measured against the
    norm of another field (a transverse momentum against the streamwise one,
    whose size sets the rounding of the shared fluxes)."""
    scale = scale or {}
    for name in names:
        a = to_host(ss.variables[name].data)
        b = so.variables[name].data
        if name in scale:
            ref = so.variables[scale[name]].data
            e = numpy.linalg.norm((a - b).ravel()) / numpy.linalg.norm(ref.ravel())
        else:
            e = rel_l2(a, b)
        assert e <= tol, (name, e)


def test_advection3d_config_matches_oracle(oracle):
    """64^3 periodic advection with the compact filter after every stage,
    dt = 1e-3, 100 RK steps: the FP64 path matches the oracle to 1e-12."""
    from pyranda_gb300 import pyrandaSim, problems
    ss = problems.build_advection3d(pyrandaSim, 64, silent=True)
    so = problems.build_advection3d(oracle.OracleSim, 64)
    t = to = 0.0
    for _ in range(100):
        t = ss.rk4(t, 1.0e-3)
        to = so.rk4(to, 1.0e-3)
    _fields_match(ss, so, ["phi"])
    # the blob has moved: the solution differs from the initial condition
    assert rel_l2(to_host(ss.variables["phi"].data), to_host(ss.variables["phi0"].data)) > 1e-3


def test_laplacian_d4_and_tensor_divergence_in_the_eom(oracle):
    """lap(), dd4x/y/z() and divT() of the EOM language (pyranda.py:818-835) against the oracle."""
    from pyranda_gb300 import pyrandaSim
    mesh = "xdom = (0.0, 1.0, 24)\nydom = (0.0, 0.9375, 16, periodic=True)\nzdom = (0.0, 0.9, 10, periodic=True)"
    eom = """
:lp: = lap(:f:)
:d4x: = dd4x(:f:)
:d4y: = dd4y(:g:)
:d4z: = dd4z(:f:)
[:tx:,:ty:,:tz:] = divT(:f:,:g:,:f:,:g:,:f:,:g:,:f:,:g:,:f:)
"""
    ic = ":f: = sin(2*pi*meshy)*exp(meshx) + cos(2*pi*meshz)\n:g: = meshx*meshx*cos(2*pi*meshy)"
    ss = pyrandaSim("ops", mesh, silent=True)
    so = oracle.OracleSim("ops", mesh)
    for s in (ss, so):
        s.EOM(eom)
        s.setIC(ic)
        s.updateVars()
    _fields_match(ss, so, ["lp", "d4x", "d4y", "d4z", "tx", "ty", "tz"])


def _packs(ss):
    from pyranda_gb300 import pyrandaBC, pyrandaTimestep
    ss.addPackage(pyrandaBC(ss))
    ss.addPackage(pyrandaTimestep(ss))


def test_shock_interface_small_matches_oracle(oracle):
    """The shock-interface problem (one-sided x closures, periodic y/z, LAD,
    extrapolation BCs) on a 64x16x16 grid: 5 steps match the oracle."""
    from pyranda_gb300 import pyrandaSim, problems
    ss = problems.build_shock(pyrandaSim, 64, 16, 16, _packs, silent=True)
    so = problems.build_shock(oracle.OracleSim, 64, 16, 16, lambda s: (s.addPackage("BC"), s.addPackage("Timestep")))
    t = to = 0.0
    for _ in range(5):
        dt = float(ss.variables["dt"].data) * 0.5
        dto = so.variables["dt"].data * 0.5
        assert abs(dt - dto) <= 1e-12 * dto
        t = ss.rk4(t, dt)
        to = so.rk4(to, dto)
    _fields_match(ss, so, ["rho", "rhou", "rhov", "rhow", "Et", "u", "p", "mu"],
                  scale={"rhov": "rhou", "rhow": "rhou"})


def test_shock_interface_full_size_runs():
    """The 512x128x128 shock-interface configuration steps on one GPU in both
    precisions and keeps density and pressure positive."""
    from pyranda_gb300 import pyrandaSim, problems
    for prec in ("fp64", "fp32"):
        ss = problems.build_shock(pyrandaSim, 512, 128, 128, _packs, silent=True, precision=prec)
        ss.use_graphs(True)
        t = 0.0
        for _ in range(4):
            t = ss.rk4(t, ss.variables["dt"].data * 0.5)
        rho, p = ss.variables["rho"].data, ss.variables["p"].data
        assert bool(torch.isfinite(ss.variables["Et"].data).all())
        assert float(rho.min()) > 0.5 and float(p.min()) > 0.5
        del ss
        torch.cuda.empty_cache()


def test_restart_round_trip(tmp_path, monkeypatch):
    """A run interrupted by writeRestart / pyrandaRestart continues bit for bit."""
    from pyranda_gb300 import pyrandaRestart, pyrandaSim, pyrandaTimestep
    from pyranda_gb300.problems import build_tgv
    monkeypatch.chdir(tmp_path)
    a = build_tgv(pyrandaSim, 24, lambda s: s.addPackage(pyrandaTimestep(s)), silent=True)
    t = 0.0
    for _ in range(3):
        t = a.rk4(t, a.variables["dt"].data * 0.5)
    a.writeRestart(ivars={"note": "x", "arr": numpy.arange(3.0)})
    [b, local] = pyrandaRestart(a.name)
    assert local["note"] == "x" and numpy.array_equal(local["arr"], numpy.arange(3.0))
    assert b.cycle == a.cycle and b.time == pytest.approx(float(t))
    ta, tb = float(t), float(b.time)
    for _ in range(2):
        ta = a.rk4(ta, a.variables["dt"].data * 0.5)
        tb = b.rk4(tb, b.variables["dt"].data * 0.5)
    for name in ("rho", "rhou", "rhov", "rhow", "Et"):
        assert torch.equal(a.variables[name].data, b.variables[name].data), name


def test_vtk_dump(tmp_path, monkeypatch):
    """sim.write() (pyranda.py:431-470): pyranda's binary VTK dump of the device fields and the .visit list."""
    from pyranda_gb300 import problems, pyrandaSim
    monkeypatch.chdir(tmp_path)
    ss = problems.build_tgv(pyrandaSim, 16, _ts, silent=True)
    ss.rk4(0.0, ss.variables["dt"].data.clone())
    path = ss.write(["rho", "u"])
    assert os.path.basename(path) == "proc-000000.0000001.vtk"
    raw = open(path, "rb").read()
    assert b"DIMENSIONS  16 16 16  \n" in raw
    nb = 16 ** 3 * 4

    def block(name):
        tag = b"SCALARS %s float \nLOOKUP_TABLE default \n" % name.encode()
        p = raw.index(tag) + len(tag)
        return numpy.frombuffer(raw[p:p + nb], dtype=">f4")

    rho, u = block("rho"), block("u")
    tag = b"SCALARS u float \nLOOKUP_TABLE default \n"
    assert len(raw) == raw.index(tag) + len(tag) + nb
    assert numpy.array_equal(rho, to_host(ss.variables["rho"].data).ravel(order="F").astype(numpy.float32))
    assert numpy.array_equal(u, to_host(ss.variables["u"].data).ravel(order="F").astype(numpy.float32))
    visit = open(os.path.join("TGvortex", "pyranda.visit")).read()
    assert visit.startswith("!NBLOCKS 1 \n!TIME ") and "vis0000001/proc-000000.0000001.vtk" in visit


GOLDEN_DIR = os.path.join(os.path.dirname(__file__), "golden")


def _oracle_bc_ts(s):
    s.addPackage("BC")
    s.addPackage("Timestep")


@pytest.mark.parametrize("n", [64, 128])
def test_euler_2d_profile_golden(oracle, n):
    """tests/cases/test2deuler.py euler-2d-N (examples/euler.py): the GPU
    pyrandaSim reproduces the reference's density profile within the
    reference's tolerance (tests/testObj.py:checkProfile < 1e-4), and the
    oracle's profile to rounding."""
    from pyranda_gb300 import pyrandaSim
    path = os.path.join(GOLDEN_DIR, "euler-2d-%d.dat" % n)
    x, rho = scripts.euler_2d(pyrandaSim, n, _bc_ts, silent=True)
    err = scripts.profile_error(path, x, rho)
    assert err < 1.0e-4, err
    xo, ro = scripts.euler_2d(oracle.OracleSim, n, _oracle_bc_ts)
    diff = float(numpy.abs(rho - ro).max() / numpy.abs(ro).max())
    print("euler-2d-%d: profile error %.2e, max difference from the oracle %.2e" % (n, err, diff))
    assert diff <= 1e-10, diff


def test_kelvin_helmholtz_2d_profile_golden(oracle):
    """tests/cases/test2deuler.py KH-2d-64 (examples/KH.py): AFLES terms,
    courant and diffusion limits, grad(T): the reference's density profile at
    t = 1.5 within its tolerance, and the oracle's profile to rounding."""
    from pyranda_gb300 import pyrandaSim
    path = os.path.join(GOLDEN_DIR, "KelvinHelmholtzKH-2d-64.dat")
    x, rho = scripts.kelvin_helmholtz_2d(pyrandaSim, 64, _bc_ts, silent=True)
    err = scripts.profile_error(path, x, rho)
    assert err < 1.0e-4, err
    xo, ro = scripts.kelvin_helmholtz_2d(oracle.OracleSim, 64, _oracle_bc_ts)
    diff = float(numpy.abs(rho - ro).max() / numpy.abs(ro).max())
    print("KH-2d-64: profile error %.2e, max difference from the oracle %.2e" % (err, diff))
    assert diff <= 1e-9, diff


def test_tgv_256_fp64_step_matches_oracle(oracle):
    """The benchmark's workload itself: the 256^3 Taylor-Green vortex at
    Mach 0.1 / Re 1600 on the plain FP64 path.  The time step and every field
    after one RK step (five stages, each with the filters, LAD ring operators
    and the courant / diffusion limits) match the oracle, run on every host
    core, to relative L2 <= 1e-12."""
    from pyranda_gb300 import pyrandaSim, problems
    oracle.set_threads(os.cpu_count() or 1)
    ss = problems.build_tgv(pyrandaSim, 256, _ts, ns=True, silent=True)
    so = problems.build_tgv(oracle.OracleSim, 256, lambda s: s.addPackage("Timestep"), ns=True)
    dt = float(ss.variables["dt"].data) * 0.5
    dto = float(so.variables["dt"].data) * 0.5
    assert abs(dt - dto) <= 1e-13 * dto
    ss.rk4(0.0, dt)
    so.rk4(0.0, dto)
    _fields_match(ss, so, ["rho", "rhou", "rhov", "rhow", "Et", "u", "p", "mu", "enst"], scale={"rhow": "rhou"})
    dtn, dton = float(ss.variables["dt"].data), float(so.variables["dt"].data)
    assert abs(dtn - dton) <= 1e-12 * dton
    # beta = gbar(|ring(div)| rho) * 7e-3.  The TGV dilatation div = ux + vy + wz
    # cancels to a small remainder of O(1) terms, and ring() takes its 8th
    # derivative, which amplifies the rounding of that remainder.  So: div
    # agrees to 1e-12 relative to the terms it is made of, and beta agrees to
    # 1e-12 with the oracle's operators applied to the GPU's own div.
    div_g = to_host(ss.variables["div"].data)
    ux = so.variables["ux"].data
    assert numpy.linalg.norm((div_g - so.variables["div"].data).ravel()) <= 1e-12 * numpy.linalg.norm(ux.ravel())
    og = so.grid
    beta_ref = og.gfilter(numpy.abs(og.ring(div_g, 2)) * so.variables["rho"].data) * 7.0e-3
    e = rel_l2(to_host(ss.variables["beta"].data), beta_ref)
    assert e <= 1e-12, e


def test_shock_interface_full_size_step_matches_oracle(oracle):
    """The 512x128x128 shock-interface configuration (one-sided x closures,
    periodic y/z, LAD, extrapolation BCs) on the plain FP64 path: one RK step
    matches the oracle to relative L2 <= 1e-12."""
    from pyranda_gb300 import pyrandaSim, problems
    oracle.set_threads(os.cpu_count() or 1)
    ss = problems.build_shock(pyrandaSim, 512, 128, 128, _packs, silent=True)
    so = problems.build_shock(oracle.OracleSim, 512, 128, 128, _oracle_bc_ts)
    dt = float(ss.variables["dt"].data) * 0.5
    dto = float(so.variables["dt"].data) * 0.5
    assert abs(dt - dto) <= 1e-12 * dto
    ss.rk4(0.0, dt)
    so.rk4(0.0, dto)
    _fields_match(ss, so, ["rho", "rhou", "rhov", "rhow", "Et", "u", "p", "mu"],
                  scale={"rhov": "rhou", "rhow": "rhou"})


def test_euler_rz_profile_golden(oracle):
    """tests/cases/test2deuler.py euler-RZ-128 (examples/eulerRZ.py): the GPU
    pyrandaSim on a cylindrical mesh with a symmetry plane at the axis
    reproduces the reference's pressure profile within its tolerance, and the
    oracle's profile to rounding."""
    from pyranda_gb300 import pyrandaSim, pyrandaBC
    path = os.path.join(GOLDEN_DIR, "euler-RZ-128.dat")
    x, p = scripts.euler_rz(pyrandaSim, 128, lambda s: s.addPackage(pyrandaBC(s)), silent=True)
    err = scripts.profile_error(path, x, p)
    assert err < 1.0e-4, err
    xo, po = scripts.euler_rz(oracle.OracleSim, 128, lambda s: s.addPackage("BC"))
    diff = float(numpy.abs(p - po).max() / numpy.abs(po).max())
    print("euler-RZ-128: profile error %.2e, max difference from the oracle %.2e" % (err, diff))
    assert diff <= 1e-10, diff


@pytest.mark.parametrize("name,run", [
    ("euler-SPH-1D", lambda S, pk: scripts.euler_sph_1d(S, 128, pk, silent=True)),
    ("euler-SPH-2D", lambda S, pk: scripts.euler_sph_2d(S, 32, pk, silent=True)),
    ("cylinder_omesh-2d-64", lambda S, pk: scripts.cylinder_omesh(S, 64, pk, silent=True)),
])
def test_spherical_and_curvilinear_profile_goldens(name, run):
    """tests/cases/test2deuler.py euler-SPH-1D / euler-SPH-2D and
    tests/cases/testCylinder.py cylinder_omesh-2d-64: the GPU pyrandaSim on
    spherical grids and on a curvilinear O-mesh (supplied coordinates, metric
    div, slip wall with the metric normal, curvilinear courant limit)
    reproduces the reference's profiles within the reference's tolerance 1e-4
    and, as the oracle reproduces each file to 1e-13, to 1e-8 -- rounding
    differences grown over 256 to 1025 RK steps."""
    from pyranda_gb300 import pyrandaSim
    path = os.path.join(GOLDEN_DIR, name + ".dat")
    x, v = run(pyrandaSim, _bc_ts)
    assert numpy.abs(x - numpy.loadtxt(path)[0]).max() < 1e-12
    err = scripts.profile_error(path, x, v)
    print("%s: profile error %.2e" % (name, err))
    assert err < 1.0e-4, err
    assert err < 1.0e-8, err


@pytest.mark.parametrize("n", [16, 64, 256])
def test_heat_1d_golden(n):
    """tests/cases/testHeat1D.py heat1D-analytic-N on the GPU: the Laplacian's
    one-sided c10d2 rows with bc.const ends keep the linear steady state
    (golden 0.0, absolute tolerance 1e-4; rounding only here)."""
    from pyranda_gb300 import pyrandaSim, pyrandaBC
    err = scripts.heat_1d(pyrandaSim, n, lambda s: s.addPackage(pyrandaBC(s)), silent=True)
    assert GOLD["heat1D-analytic-%d" % n]["value"] == 0.0
    assert err < 1e-10, err


@pytest.mark.parametrize("n", [25, 50, 100, 200])
def test_integration_golden(n):
    """tests/cases/testIntegration.py integration-N on the GPU: the LSRK(5,4)
    update and its stage times on one point.  (N = 400 is left to the oracle:
    its summed error, 5e-11, is at the rounding level of the 400 steps.)"""
    from pyranda_gb300 import pyrandaSim
    _close(scripts.integration(pyrandaSim, n, silent=True), "integration-%d" % n)


def test_curvilinear_restart_round_trip(tmp_path, monkeypatch):
    """A curvilinear run (an O-mesh from a mesh function) interrupted by
    writeRestart / pyrandaRestart: the restart rebuilds the metrics from the
    coordinates it holds (pyranda.py:1064-1069), bit for bit, and the run
    continues to rounding (scalar variables keep their Python-number or
    device-scalar type, which sets how torch divides by them)."""
    from pyranda_gb300 import pyrandaRestart, pyrandaSim
    monkeypatch.chdir(tmp_path)
    NX = NY = 24

    def cyl_mesh(i, j, k):
        theta = float(i) / float(NX) * 2.0 * numpy.pi
        r = float(j) / float(NY - 1) * 9.0 + 1.0
        return r * numpy.cos(theta), r * numpy.sin(theta), 0.0

    opts = {"coordsys": 3, "function": cyl_mesh, "periodic": [True, False, False], "periodicGrid": False,
            "x1": [0.0, 0.0, 0.0], "xn": [1.0, 1.0, 1.0], "nn": [NX, NY, 1]}
    a = pyrandaSim("omesh_restart", opts, silent=True)
    _bc_ts(a)
    u0 = numpy.sqrt(1.4) * 1.5
    a.EOM(scripts.OMESH_EOM.replace("u0", str(u0)).replace("p0", "1.0").replace("rho0", "1.0"))
    a.setIC(scripts.OMESH_IC.replace("mach", "1.5"))
    dt = float(a.variables["dt"].data) * 0.08
    t = 0.0
    for _ in range(2):
        t = a.rk4(t, dt)
    a.writeRestart()
    [b, _] = pyrandaRestart(a.name)
    for name in ("dAx", "dAy", "dBx", "dBy", "dtJ", "d1", "d2"):
        assert torch.equal(a.getVar(name), b.getVar(name)), name
    ta, tb = float(t), float(b.time)
    for _ in range(2):
        ta = a.rk4(ta, dt)
        tb = b.rk4(tb, dt)
    exact = True
    for name in ("rho", "rhou", "rhov", "Et", "u", "v"):
        x, y = a.variables[name].data, b.variables[name].data
        exact = exact and torch.equal(x, y)
        assert float(torch.linalg.vector_norm(x - y) / torch.linalg.vector_norm(x)) <= 1e-12, name
    print("curvilinear restart: continuation bit for bit: %s" % exact)
