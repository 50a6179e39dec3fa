"""GPU parity: the CUDA path (through the C ABI) against the reference's own
outputs (golden fixtures) and the CPU oracle, at sizes the oracle runs in
seconds.

Tolerances (relative L-inf, scaled by the field's max |value|):
  * FP64 arithmetic, FP64 storage: 1e-11 -- only summation order and FMA
    contraction differ from the reference's expressions;
  * FP32 arithmetic on FP64/FP32 storage: 2e-5;
  * FP16-deviation storage: 3e-3.
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import load_golden, rel_err
from oracle import oracle as O

import cflbm
from cflbm import Batch, Solver
from cflbm import _lib as C

pytestmark = pytest.mark.gpu

TOL64 = 1e-11


def ref2d_gpu(nx, ny, tau0, u0, ran, steps, **kw):
    with Solver(lattice=9, nx=nx, ny=ny, profile="ref2d", tau0=tau0, u0=u0, ref_ran=ran,
                **kw) as s:
        s.step(steps)
        u, v, w, p = s.macros()
        return dict(u=u[0], v=v[0], p=p[0], fpost=s.get_f()[:, 0], force=s.force_history(),
                    cdcl=s.forces()[1])


def ref3d_gpu(nx, ny, nz, tau0, u0, ran, steps, **kw):
    with Solver(lattice=27, nx=nx, ny=ny, nz=nz, profile="ref3d", tau0=tau0, u0=u0,
                ref_ran=ran, **kw) as s:
        s.step(steps)
        u, v, w, p = s.macros()
        return dict(u=u, v=v, w=w, p=p, fpost=s.get_f())


def test_ref2d_matches_reference_golden(cuda):
    g = load_golden("ref2d_96x40")
    m = g["meta"]
    r = ref2d_gpu(m["nx"], m["ny"], m["tau0"], m["u0"], g["ran"], m["steps"])
    for k in ("u", "v", "p", "fpost"):
        assert rel_err(r[k], g[k]) < TOL64, k
    u0, nx = m["u0"], m["nx"]
    cd = 2.0 * r["force"][:, 0] / u0 / u0 / 0.03125 / (nx - 1)
    cl = 2.0 * r["force"][:, 1] / u0 / u0 / 0.03125 / (nx - 1)
    assert r["force"].shape[0] == m["steps"]
    assert rel_err(cd, g["cdcl"][:, 0]) < 1e-10
    assert rel_err(cl, g["cdcl"][:, 1]) < 1e-9
    assert abs(r["cdcl"][0] - g["cdcl"][-1, 0]) < 1e-10 * abs(g["cdcl"][-1, 0])


def test_ref3d_matches_reference_golden(cuda):
    g = load_golden("ref3d_40x12x12")
    m = g["meta"]
    r = ref3d_gpu(m["nx"], m["ny"], m["nz"], m["tau0"], m["u0"], g["ran"], m["steps"])
    for k in ("u", "v", "w", "p", "fpost"):
        assert rel_err(r[k], g[k]) < TOL64, k


def test_ref2ds_matches_reference_golden(cuda):
    """The serial "Kokkos/" variant (its own geometry, perturbation and wall
    rows without corners) against the compiled reference's outputs."""
    g = load_golden("ref2ds_96x36")
    m = g["meta"]
    with Solver(lattice=9, nx=m["nx"], ny=m["ny"], profile="ref2ds", tau0=m["tau0"],
                u0=m["u0"], ref_ran=g["ran"]) as s:
        s.step(m["steps"])
        u, v, w, p = s.macros()
        fstream = s.get_f_stream()[:, 0]
        fpost = s.get_f()[:, 0]
    assert rel_err(u[0], g["u"]) < TOL64
    assert rel_err(v[0], g["v"]) < TOL64
    assert rel_err(p[0], g["p"]) < TOL64
    assert rel_err(fpost, g["fpost"]) < TOL64
    assert rel_err(fstream, g["fstream"]) < TOL64


@pytest.mark.parametrize("compute,tol", [("fp64", 1e-10), ("df64", 1e-9), ("fp32", 2e-5)])
def test_ref2ds_matches_oracle_longer_run(cuda, compute, tol):
    nx, ny, steps = 240, 64, 300
    ran = np.random.default_rng(11).integers(0, 100, size=(nx + 4, ny + 4)).astype(np.int32)
    o = O.ref2ds(nx, ny, 0.03, 0.06, ran, steps)
    with Solver(lattice=9, nx=nx, ny=ny, profile="ref2ds", tau0=0.03, u0=0.06, ref_ran=ran,
                compute=compute) as s:
        s.step(steps)
        u, v, w, p = s.macros()
    sl = (slice(2, 2 + nx), slice(2, 2 + ny))
    assert rel_err(u[0], o["u"][sl].T) < tol
    assert rel_err(v[0], o["v"][sl].T) < tol
    # p is the deviation of sum(f)/3 from rest, ~4e-3 here: its error is bounded
    # on the scale of the pressure itself (1/3), which FP32 rounds at ~2e-8
    # per step, not on the deviation's own small maximum
    assert np.max(np.abs(p[0] - o["p"][sl].T)) < tol * (1.0 / 3.0)


def test_ref2d_matches_oracle_longer_run(cuda):
    nx, ny, steps = 256, 72, 600
    ran = np.random.default_rng(7).integers(0, 100, size=(nx + 4, ny + 4)).astype(np.int32)
    o = O.ref2d(nx, ny, 0.03, 0.05, ran, steps)
    r = ref2d_gpu(nx, ny, 0.03, 0.05, ran, steps)
    sl = (slice(2, 2 + nx), slice(2, 2 + ny))
    assert rel_err(r["u"], o["u"][sl].T) < 1e-10
    assert rel_err(r["v"], o["v"][sl].T) < 1e-10
    assert rel_err(r["p"], o["p"][sl].T) < 1e-10
    assert rel_err(r["force"][:, :2], o["force"]) < 1e-9


def test_ref3d_matches_oracle(cuda):
    nx, ny, nz, steps = 72, 20, 24, 40
    ran = np.random.default_rng(3).integers(0, 100, size=(nx + 6, ny + 6, nz + 6)).astype(np.int32)
    o = O.ref3d(nx, ny, nz, 0.0192, 0.04, ran, steps, want_f=True)
    r = ref3d_gpu(nx, ny, nz, 0.0192, 0.04, ran, steps)
    sl = (slice(3, 3 + nx), slice(3, 3 + ny), slice(3, 3 + nz))
    for k in ("u", "v", "w", "p"):
        assert rel_err(r[k], o[k][sl].transpose(2, 1, 0)) < 1e-10, k
    assert rel_err(r["fpost"], o["fpost"][(slice(None),) + sl].transpose(0, 3, 2, 1)) < 1e-10


CHANNEL_CASES = {
    # 2-D cylinder, free-slip walls (the small benchmark problem, scaled down)
    "d2q9_cyl_freeslip": dict(lattice=9, nx=160, ny=41, nz=1, tau0=0.03, u0=0.05,
                              wall_y="freeslip", geom="cylinder", cx=32, cy=20, diam=10),
    "d2q9_cyl_noslip": dict(lattice=9, nx=96, ny=33, nz=1, tau0=0.08, u0=0.05,
                            wall_y="noslip", geom="cylinder", cx=24, cy=15, diam=7),
    "d2q9_periodic": dict(lattice=9, nx=64, ny=32, nz=1, tau0=0.05, u0=0.04,
                          wall_y="periodic", geom="cylinder", cx=20, cy=11, diam=6),
    # 3-D spanwise cylinder, free-slip y, periodic z
    "d3q27_cyl": dict(lattice=27, nx=64, ny=32, nz=12, tau0=0.0192, u0=0.04,
                      wall_y="freeslip", wall_z="periodic", geom="cylinder", cx=16, cy=16,
                      diam=8),
    # 3-D sphere, free-slip on all side faces
    "d3q27_sphere": dict(lattice=27, nx=48, ny=24, nz=24, tau0=0.0192, u0=0.03,
                         wall_y="freeslip", wall_z="freeslip", geom="sphere", cx=14, cy=12,
                         cz=12, diam=9),
    # 3-D no-slip box walls
    "d3q27_noslip": dict(lattice=27, nx=40, ny=18, nz=16, tau0=0.05, u0=0.03,
                         wall_y="noslip", wall_z="noslip", geom="sphere", cx=12, cy=9,
                         cz=8, diam=6),
    # narrower than one 32-cell tile, at the smallest y / z extents (4 cells)
    "d2q9_narrow": dict(lattice=9, nx=20, ny=5, nz=1, tau0=0.05, u0=0.04,
                        wall_y="noslip", geom="cylinder", cx=6, cy=2, diam=2.5),
    "d3q27_narrow": dict(lattice=27, nx=21, ny=4, nz=4, tau0=0.05, u0=0.03,
                         wall_y="periodic", wall_z="freeslip", geom="sphere", cx=7, cy=2,
                         cz=2, diam=2.5),
}


def oracle_channel(case, steps, alpha=None):
    c = dict(case)
    wall = {"freeslip": O.WALL_FREESLIP, "noslip": O.WALL_NOSLIP, "periodic": O.WALL_PERIODIC}
    geom = {"none": O.GEOM_NONE, "cylinder": O.GEOM_CYLINDER, "sphere": O.GEOM_SPHERE}
    cfg = O.channel_cfg(c["lattice"], c["nx"], c["ny"], c["nz"], tau0=c["tau0"], u_in=c["u0"],
                        wall_y=wall[c.get("wall_y", "freeslip")],
                        wall_z=wall[c.get("wall_z", "periodic")], geom=geom[c["geom"]],
                        cx=c.get("cx", 0), cy=c.get("cy", 0), cz=c.get("cz", 0),
                        diam=c.get("diam", 0), amp=1e-3, seed=1234, alpha=alpha)
    return O.channel(cfg, steps)


def gpu_channel(case, steps, **kw):
    with Solver(perturb_amp=1e-3, seed=1234, **case, **kw) as s:
        s.step(steps)
        u, v, w, p = s.macros()
        return dict(u=u, v=v, w=w, p=p, fpost=s.get_f(), force=s.force_history(), solver_info=s.info())


@pytest.mark.parametrize("name", sorted(CHANNEL_CASES))
def test_channel_fp64_matches_oracle(cuda, name):
    case = CHANNEL_CASES[name]
    steps = 300 if case["lattice"] == 9 else 40
    o = oracle_channel(case, steps)
    r = gpu_channel(case, steps)
    for k in ("u", "v", "w", "p", "fpost"):
        if k == "w" and case["lattice"] == 9:
            continue
        assert rel_err(r[k], o[k]) < TOL64 * 10, (name, k)
    assert rel_err(r["force"], o["force"]) < 1e-9, name


@pytest.mark.parametrize("name", ["d2q9_cyl_freeslip", "d3q27_cyl", "d3q27_sphere"])
def test_channel_fp64_stays_at_roundoff(cuda, name):
    """Over a few steps FP64 arithmetic stays at round-off from the oracle: the
    moments' cascade and the relaxation's Horner form per +/- pair change only
    the order of FP64 operations.  One step's arithmetic in FP32 would show at
    ~1e-7."""
    case = CHANNEL_CASES[name]
    o = oracle_channel(case, 5)
    r = gpu_channel(case, 5)
    for k in ("u", "v", "w", "p", "fpost"):
        if k == "w" and case["lattice"] == 9:
            continue
        assert rel_err(r[k], o[k]) < 1e-12, (name, k)
    assert rel_err(r["force"], o["force"]) < 1e-12, name


@pytest.mark.parametrize("name", sorted(CHANNEL_CASES))
def test_channel_df64_matches_oracle(cuda, name):
    """Double-float collision (pairs of FP32, about 48 bits) on FP64 storage stays
    within 1e-9 of the FP64 oracle (FP32 collision: 2e-5)."""
    case = CHANNEL_CASES[name]
    steps = 300 if case["lattice"] == 9 else 40
    o = oracle_channel(case, steps)
    r = gpu_channel(case, steps, storage="fp64", compute="df64")
    for k in ("u", "v", "w", "p", "fpost"):
        if k == "w" and case["lattice"] == 9:
            continue
        assert rel_err(r[k], o[k]) < 1e-9, (name, k)
    assert rel_err(r["force"], o["force"]) < 1e-8, name


def test_reference_profiles_df64_close_to_fp64(cuda):
    g = load_golden("ref2d_96x40")
    m = g["meta"]
    a = ref2d_gpu(m["nx"], m["ny"], m["tau0"], m["u0"], g["ran"], m["steps"])
    b = ref2d_gpu(m["nx"], m["ny"], m["tau0"], m["u0"], g["ran"], m["steps"], compute="df64")
    for k in ("u", "v", "p", "fpost", "force"):
        assert rel_err(b[k], a[k]) < 1e-10, k
    nx, ny, nz = 40, 14, 16
    ran = np.random.default_rng(3).integers(0, 100, size=(nx + 6, ny + 6, nz + 6)).astype(np.int32)
    a = ref3d_gpu(nx, ny, nz, 0.0192, 0.04, ran, 30)
    b = ref3d_gpu(nx, ny, nz, 0.0192, 0.04, ran, 30, compute="df64")
    for k in ("u", "v", "w", "p", "fpost"):
        assert rel_err(b[k], a[k]) < 1e-10, k


def test_df64_needs_fp64_storage(cuda):
    with pytest.raises(cflbm.CflbmError):
        Solver(storage="fp32", compute="df64", **CHANNEL_CASES["d2q9_cyl_freeslip"])


@pytest.mark.parametrize("storage,compute,tol", [("fp64", "fp32", 2e-5), ("fp32", "fp32", 2e-5),
                                                 ("fp32", "fp64", 2e-5),
                                                 ("fp16dev", "fp32", 3e-3)])
def test_channel_reduced_precision_close_to_oracle(cuda, storage, compute, tol):
    # every wall combination: listed tiles pull through the face-state tables
    for name in sorted(CHANNEL_CASES):
        case = CHANNEL_CASES[name]
        steps = 200 if case["lattice"] == 9 else 30
        o = oracle_channel(case, steps)
        r = gpu_channel(case, steps, storage=storage, compute=compute)
        assert rel_err(r["u"], o["u"]) < tol, (name, storage, compute)
        assert rel_err(r["v"], o["v"]) < 20 * tol, (name, storage, compute)
        assert rel_err(r["force"][:, 0], o["force"][:, 0]) < 10 * tol, (name, storage, compute)


@pytest.mark.parametrize("name", sorted(CHANNEL_CASES))
def test_one_cell_and_pair_kernels_agree_bit_for_bit(cuda, name):
    """FP32 collision on FP64 storage (one cell per thread) and on FP32 storage
    (two cells per thread, packed FP32x2) hold the same FP32 values every step,
    listed tiles included, so states and forces must be identical."""
    case = CHANNEL_CASES[name]
    steps = 60 if case["lattice"] == 9 else 12
    a = gpu_channel(case, steps, storage="fp64", compute="fp32")
    b = gpu_channel(case, steps, storage="fp32", compute="fp32")
    assert np.array_equal(a["fpost"], b["fpost"]), name
    assert np.array_equal(a["force"], b["force"]), name
    assert np.array_equal(a["u"], b["u"]), name


@pytest.mark.parametrize("storage,tol", [("fp32", 2e-5), ("fp16dev", 3e-3)])
def test_wide_d2q9_grid_close_to_oracle(cuda, storage, tol):
    """D2Q9 grids of 2^20 cells and more take the 48-register pair kernel; it
    must agree with the oracle as the other FP32-collision forms do, and bit for
    bit with the same channel advanced as a one-instance batch (same cell code,
    other kernels)."""
    case = dict(lattice=9, nx=1024, ny=1024, nz=1, tau0=0.03, u0=0.05, wall_y="freeslip",
                geom="cylinder", cx=200, cy=512, diam=64)
    steps = 20
    o = oracle_channel(case, steps)
    r = gpu_channel(case, steps, storage=storage, compute="fp32")
    assert rel_err(r["u"], o["u"]) < tol
    assert rel_err(r["v"], o["v"]) < 20 * tol
    assert rel_err(r["force"][:, 0], o["force"][:, 0]) < 10 * tol
    with Batch([dict(case, perturb_amp=1e-3, seed=1234, storage=storage, compute="fp32")],
               graph_steps=8, autotune=False, tile_height=4, blocks_per_sm=0) as b:
        b.step(steps)
        b.synchronize()
        assert np.array_equal(b.instance(0).get_f(), r["fpost"])


def test_brinkman_porosity_matches_oracle(cuda):
    case = dict(CHANNEL_CASES["d2q9_cyl_freeslip"])
    rng = np.random.default_rng(11)
    alpha = np.zeros((1, case["ny"], case["nx"]))
    alpha[0, 5:35, 60:100] = rng.uniform(0, 1, size=(30, 40))
    o = oracle_channel(case, 150, alpha=alpha)
    r = gpu_channel(case, 150, alpha=alpha)
    for k in ("u", "v", "p", "fpost"):
        assert rel_err(r[k], o[k]) < 1e-6, k  # alpha is stored as FP32 on the GPU


def test_steps_are_deterministic_and_resumable(cuda):
    case = CHANNEL_CASES["d3q27_cyl"]
    with Solver(perturb_amp=1e-3, **case) as a, Solver(perturb_amp=1e-3, **case) as b:
        a.step(17)
        b.step(10)
        f10 = b.get_f()
        b.set_f(f10, steps_done=10)
        b.step(7)
        assert np.array_equal(a.get_f(), b.get_f())
        assert np.array_equal(a.macros()[0], b.macros()[0])
        assert a.info().steps_done == b.info().steps_done == 17


@pytest.mark.parametrize("name", ["d2q9_cyl_freeslip", "d3q27_cyl", "d3q27_noslip"])
@pytest.mark.parametrize("storage", ["fp64", "fp32", "fp16dev", "fp16dev-sr"])
def test_layouts_give_identical_states(cuda, name, storage):
    """Every kernel (register-fed pairs, line-staged rows, one-cell listed
    tiles) rounds a state alike, FP16 stochastic rounding included."""
    case = CHANNEL_CASES[name]
    steps = 60 if case["lattice"] == 9 else 12
    rounding = "stochastic" if storage.endswith("-sr") else "nearest"
    out = []
    for layout in ("soa", "rows"):
        with Solver(perturb_amp=1e-3, layout=layout, storage=storage.split("-")[0],
                    compute="fp32", rounding=rounding, **case) as s:
            s.step(steps)
            out.append((s.get_f(), s.force_history()))
    assert np.array_equal(out[0][0], out[1][0])
    assert np.array_equal(out[0][1], out[1][1])


@pytest.mark.parametrize("name", ["d3q27_cyl", "d3q27_noslip"])
@pytest.mark.parametrize("rounding", ["stochastic", "nearest"])
def test_line_staged_sweep_matches_pair_kernel(cuda, name, rounding, monkeypatch):
    """The opt-in line-staged FP16 sweep (CFLBM_FP16_SWEEP=lines, read when a
    handle is created) gives the register-fed pair kernel's states and forces
    bit for bit, no-slip faces and solid links included."""
    case = CHANNEL_CASES[name]
    out = []
    for mode in ("registers", "lines"):
        monkeypatch.setenv("CFLBM_FP16_SWEEP", mode)
        with Solver(perturb_amp=1e-3, layout="rows", storage="fp16dev", compute="fp32",
                    rounding=rounding, **case) as s:
            s.step(12)
            s.synchronize()
            out.append((s.get_f(), s.force_history()))
    assert np.array_equal(out[0][0], out[1][0])
    assert np.array_equal(out[0][1], out[1][1])


def test_reference_profile_rows_layout_matches_golden(cuda):
    g = load_golden("ref3d_40x12x12")
    m = g["meta"]
    r = ref3d_gpu(m["nx"], m["ny"], m["nz"], m["tau0"], m["u0"], g["ran"], m["steps"],
                  layout="rows")
    for k in ("u", "v", "w", "p", "fpost"):
        assert rel_err(r[k], g[k]) < TOL64, k


def test_mass_and_momentum_sums(cuda):
    case = CHANNEL_CASES["d2q9_cyl_freeslip"]
    o = oracle_channel(case, 50)
    with Solver(perturb_amp=1e-3, seed=1234, **case) as s:
        s.step(50)
        mass, mom = s.mass()
    fl = (O.channel_mask(O.channel_cfg(9, case["nx"], case["ny"], geom=O.GEOM_CYLINDER,
                                       cx=case["cx"], cy=case["cy"], diam=case["diam"])) == 0)
    ref_mass = float(np.sum((1.0 + o["fpost"].sum(0))[fl]))
    assert abs(mass - ref_mass) < 1e-10 * ref_mass
    e, _, _ = O.lattice(9)
    ref_mx = float(np.sum(np.einsum("i,i...->...", e[:, 0], o["fpost"])[fl]))
    assert abs(mom[0] - ref_mx) < 1e-9 * abs(ref_mx)


def test_macros_device_and_tecplot_from_handle(cuda, tmp_path):
    import torch
    case = CHANNEL_CASES["d2q9_cyl_freeslip"]
    with Solver(perturb_amp=1e-3, **case) as s:
        s.step(20)
        u, v, w, p = s.macros()
        tu = torch.empty(s.shape, dtype=torch.float64, device=cuda)
        s.macros_device(tu, None, None, None)
        s.synchronize()
        assert np.array_equal(tu.cpu().numpy(), u)
        path = str(tmp_path / "h.plt")
        s.write_tecplot(path, 3)
        p2 = str(tmp_path / "f.plt")
        cflbm.solver.write_tecplot_fields(p2, u[0], v[0], None, p[0], 3)
        assert open(path, "rb").read() == open(p2, "rb").read()


def test_step_zero_macros_are_initial_fields(cuda):
    case = CHANNEL_CASES["d2q9_cyl_freeslip"]
    o = oracle_channel(case, 0)
    with Solver(perturb_amp=1e-3, seed=1234, **case) as s:
        u, v, w, p = s.macros()
    assert np.array_equal(u, o["u"])
    assert np.array_equal(v, o["v"])


def test_launches_are_counted(cuda):
    n0 = cflbm.launch_count()
    with Solver(**CHANNEL_CASES["d2q9_periodic"]) as s:
        s.step(5)
        s.synchronize()
    assert cflbm.launch_count() - n0 >= 2 * 5  # fast + resolving sweep per step


def test_forces_async_matches_forces(cuda):
    """cflbm_forces_async queues the same (Fx, Fy, Fz) that cflbm_forces returns,
    step by step, without synchronising."""
    import torch
    case = CHANNEL_CASES["d2q9_cyl_freeslip"]
    out = torch.full((6, 3), -1.0, dtype=torch.float64).pin_memory()
    with Solver(perturb_amp=1e-3, seed=1234, **case) as s:
        s.forces_async(out[0].data_ptr())  # before any step: zero
        for k in range(1, 6):
            s.step(1)
            s.forces_async(out[k].data_ptr())
        s.synchronize()
        hist = s.force_history()
        f, _ = s.forces()
    assert np.array_equal(out[0].numpy(), np.zeros(3))
    assert np.array_equal(out[1:].numpy(), hist[:5])
    assert np.array_equal(out[5].numpy(), f)


def test_bounded_wait_timeout_reaches_the_host(cuda):
    """The bounded-wait error path of the line-staged sweep, made to run out on
    purpose with an mbarrier that nothing arrives on (no copy in flight): the
    next synchronising call reports the timeout, the handle stays failed, and
    the CUDA context stays usable for a new handle."""
    case = CHANNEL_CASES["d3q27_cyl"]
    with Solver(storage="fp16dev", compute="fp32", **case) as s:
        s.step(2)
        s.synchronize()
        assert C.lib.cflbm_selftest_wait_timeout(s._h, 1000) == 0
        assert C.lib.cflbm_synchronize(s._h) != 0
        assert b"timed out" in C.lib.cflbm_last_error()
        assert C.lib.cflbm_synchronize(s._h) != 0
    with Solver(storage="fp16dev", compute="fp32", **case) as s:
        s.step(2)
        s.synchronize()
        assert np.all(np.isfinite(s.get_f()))
