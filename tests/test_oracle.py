"""CPU oracle: pinned against the reference's own outputs (golden fixtures, and
the compiled reference where it is available) and against known answers."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import load_golden
from oracle import build as obuild
from oracle import oracle as O


def test_lattice_tables():
    for Q in (9, 27):
        e, t, bb = O.lattice(Q)
        assert abs(t.sum() - 1.0) < 1e-15
        # second moment sum t e_a e_b = delta_ab / 3 (isotropy)
        m2 = np.einsum("i,ia,ib->ab", t, e, e)
        d = 2 if Q == 9 else 3
        assert np.allclose(m2[:d, :d], np.eye(d) / 3.0, atol=1e-15)
        assert np.all(e[bb] == -e)
        assert np.all(bb[bb] == np.arange(Q))


def test_ref2d_matches_reference_golden():
    g = load_golden("ref2d_96x40")
    m = g["meta"]
    o = O.ref2d(m["nx"], m["ny"], m["tau0"], m["u0"], g["ran"], m["steps"])
    G = 2
    sl = (slice(G, G + m["nx"]), slice(G, G + m["ny"]))
    # bit-for-bit: same expressions, same order, no contraction
    assert np.array_equal(o["fpost"][(slice(None),) + sl].transpose(0, 2, 1), g["fpost"])
    assert np.array_equal(o["f"][(slice(None),) + sl].transpose(0, 2, 1), g["fstream"])
    assert np.array_equal(o["u"][sl].T, g["u"])
    assert np.array_equal(o["v"][sl].T, g["v"])
    assert np.array_equal(o["p"][sl].T, g["p"])
    u0, nx = m["u0"], m["nx"]
    cd = 2.0 * o["force"][:, 0] / u0 / u0 / 0.03125 / (nx - 1)
    cl = 2.0 * o["force"][:, 1] / u0 / u0 / 0.03125 / (nx - 1)
    # test.dat holds 17 fixed decimals
    assert np.max(np.abs(cd - g["cdcl"][:, 0])) <= 6e-17 * max(1.0, np.max(np.abs(cd)))
    assert np.max(np.abs(cl - g["cdcl"][:, 1])) <= 6e-17 * max(1.0, np.max(np.abs(cl)))


def test_ref2ds_matches_reference_golden():
    """The serial "Kokkos/" variant: restatement against the compiled
    reference's own outputs, bit for bit."""
    g = load_golden("ref2ds_96x36")
    m = g["meta"]
    o = O.ref2ds(m["nx"], m["ny"], m["tau0"], m["u0"], g["ran"], m["steps"])
    G = 2
    sl = (slice(G, G + m["nx"]), slice(G, G + m["ny"]))
    assert np.array_equal(o["fpost"][(slice(None),) + sl].transpose(0, 2, 1), g["fpost"])
    assert np.array_equal(o["f"][(slice(None),) + sl].transpose(0, 2, 1), g["fstream"])
    for k in ("u", "v", "p"):
        assert np.array_equal(o[k][sl].T, g[k]), k


@pytest.mark.skipif(not obuild.reference_available(), reason="reference checkout absent")
def test_ref2ds_oracle_matches_compiled_reference_other_size():
    obuild.build_ref()
    r = O.run_ref2ds_binary(127, 47, 0.02, 0.08, 120)
    o = O.ref2ds(128, 48, 0.02, 0.08, r["ran"], 120)
    for k in ("f", "fpost", "u", "v", "p"):
        assert np.array_equal(o[k], r[k]), k


def test_ref3d_matches_reference_golden():
    g = load_golden("ref3d_40x12x12")
    m = g["meta"]
    o = O.ref3d(m["nx"], m["ny"], m["nz"], m["tau0"], m["u0"], g["ran"], m["steps"])
    G = 3
    sl = (slice(G, G + m["nx"]), slice(G, G + m["ny"]), slice(G, G + m["nz"]))
    assert np.array_equal(o["fpost"][(slice(None),) + sl].transpose(0, 3, 2, 1), g["fpost"])
    assert np.array_equal(o["f"][(slice(None),) + sl].transpose(0, 3, 2, 1), g["fstream"])
    for k in ("u", "v", "w", "p"):
        assert np.array_equal(o[k][sl].transpose(2, 1, 0), g[k]), k


@pytest.mark.skipif(not obuild.reference_available(), reason="reference checkout absent")
def test_oracle_matches_compiled_reference_other_sizes():
    obuild.build_ref()
    r = O.run_ref2d_binary(128, 48, 0.02, 0.08, 120)
    o = O.ref2d(128, 48, 0.02, 0.08, r["ran"], 120)
    for k in ("f", "fpost", "u", "v", "p"):
        assert np.array_equal(r[k], o[k]), k
    r = O.run_ref3d_binary(48, 16, 20, 0.03, 0.05, 15)
    o = O.ref3d(48, 16, 20, 0.03, 0.05, r["ran"], 15)
    for k in ("f", "fpost", "u", "v", "w", "p"):
        assert np.array_equal(r[k], o[k]), k


def test_channel_uniform_flow_is_steady():
    # No body, periodic walls: the uniform equilibrium inlet state stays uniform.
    for Q, nz in ((9, 1), (27, 6)):
        c = O.channel_cfg(Q, 24, 10, nz, tau0=0.05, u_in=0.04, wall_y=O.WALL_PERIODIC,
                          wall_z=O.WALL_PERIODIC, geom=O.GEOM_NONE, amp=0.0)
        o = O.channel(c, 30)
        assert np.max(np.abs(o["u"] - 0.04)) < 1e-15
        assert np.max(np.abs(o["v"])) < 1e-15
        assert np.max(np.abs(o["p"])) < 1e-15


def test_channel_collision_conserves_moments():
    # BGK toward the incompressible equilibrium keeps sum f = 3p and sum f e = u
    # in every fluid cell (post-collision state vs the macros it came from).
    for Q, nz in ((9, 1), (27, 8)):
        c = O.channel_cfg(Q, 40, 20, nz, tau0=0.05, u_in=0.05, wall_y=O.WALL_FREESLIP,
                          wall_z=O.WALL_PERIODIC, geom=O.GEOM_CYLINDER, cx=12, cy=10,
                          diam=6, amp=1e-3)
        o = O.channel(c, 25)
        e, t, bb = O.lattice(Q)
        fl = O.channel_mask(c) == 0
        f = o["fpost"]
        assert np.max(np.abs(f.sum(0) - 3 * o["p"])[fl]) < 1e-15
        assert np.max(np.abs(np.einsum("i,i...->...", e[:, 0], f) - o["u"])[fl]) < 1e-15
        assert np.max(np.abs(np.einsum("i,i...->...", e[:, 1], f) - o["v"])[fl]) < 1e-15


def test_channel_symmetric_body_has_no_lift():
    c = O.channel_cfg(9, 80, 41, tau0=0.05, u_in=0.05, wall_y=O.WALL_FREESLIP,
                      geom=O.GEOM_CYLINDER, cx=20, cy=20, diam=8, amp=0.0)
    o = O.channel(c, 200)
    fx, fy = o["force"][-1, 0], o["force"][-1, 1]
    assert fx > 0
    assert abs(fy) < 1e-12 * abs(fx)
    # mirror symmetry about y = 20: u even, v odd
    u, v = o["u"][0], o["v"][0]
    assert np.max(np.abs(u - u[::-1, :])) < 1e-12
    assert np.max(np.abs(v + v[::-1, :])) < 1e-12


def test_channel_perturbation_is_seeded():
    a = O.perturbation(1234, 17, 1e-3)
    assert a == O.perturbation(1234, 17, 1e-3)
    assert a != O.perturbation(1235, 17, 1e-3)
    assert -1e-3 <= a <= 1e-3
