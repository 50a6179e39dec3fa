"""Batched channels (cflbm_batch_*): every instance evolves exactly as the same
channel does alone, through graph replay and after autotuning."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import rel_err

import cflbm
from cflbm import Batch, Solver

pytestmark = pytest.mark.gpu


def configs(storage="fp32", rounding="nearest"):
    rng = np.random.default_rng(5)
    out = []
    for k in range(3):
        nx = int(rng.integers(3, 8)) * 32
        ny = int(rng.integers(2, 5)) * 32
        d = float(rng.uniform(6, 12))
        re = float(rng.uniform(40, 200))
        out.append(dict(lattice=9, nx=nx, ny=ny, tau0=3 * 0.05 * d / re, u0=0.05,
                        wall_y="freeslip", geom="cylinder", cx=nx / 4, cy=ny / 2, diam=d,
                        perturb_amp=1e-3, seed=100 + k, storage=storage, compute="fp32",
                        rounding=rounding))
    return out


def alone(cfg, steps):
    with Solver(**cfg) as s:
        s.step(steps)
        return s.get_f(), s.force_history(), s.macros()[0]


@pytest.mark.parametrize("storage", ["fp32", "fp16dev", "fp16dev-sr"])
def test_batch_instances_match_standalone_channels(cuda, storage):
    cfgs = configs(storage.split("-")[0], "stochastic" if storage.endswith("-sr") else "nearest")
    steps = 23
    with Batch(cfgs, graph_steps=6, autotune=True) as b:
        info = b.info()
        assert info.instances == 3 and info.tuned_candidates > 0
        b.step(steps)
        b.synchronize()
        for k, cfg in enumerate(cfgs):
            f_ref, h_ref, u_ref = alone(cfg, steps)
            inst = b.instance(k)
            assert inst.info().steps_done == steps
            # the same cell arithmetic in the same order: identical states; the
            # force sums run over the batch's own blocks, so their FP64
            # summation order (not the per-cell terms) differs
            assert np.array_equal(inst.get_f(), f_ref), k
            assert np.array_equal(inst.macros()[0], u_ref), k
            assert rel_err(inst.force_history(), h_ref) < 1e-12, k


def test_batch_graph_replay_equals_single_steps(cuda):
    cfgs = configs()
    with Batch(cfgs, graph_steps=4, autotune=False) as a, \
            Batch(cfgs, graph_steps=4, autotune=False) as b:
        a.step(18)          # 4 graph replays + 2 direct steps
        for _ in range(18):  # direct steps only
            b.step(1)
        for k in range(len(cfgs)):
            assert np.array_equal(a.instance(k).get_f(), b.instance(k).get_f())
            assert np.array_equal(a.instance(k).force_history(), b.instance(k).force_history())


def test_batch_instance_cannot_be_stepped_alone(cuda):
    with Batch(configs(), autotune=False) as b:
        inst = b.instance(0)
        with pytest.raises(cflbm.CflbmError):
            inst.step(1)
        with pytest.raises(IndexError):
            b.instance(5)


def test_batch_launch_shapes_agree(cuda):
    """One fast item per block (blocks_per_sm = 0) and persistent grids give the
    same states for every tile height, and the same forces for one tile height
    (force partials are per listed block, summed in block order)."""
    cfgs = configs()
    steps = 9
    ref_f = None
    for th in (1, 2, 4, 8):
        out = []
        for bps in (0, 3):
            with Batch(cfgs, graph_steps=4, autotune=False, tile_height=th,
                       blocks_per_sm=bps) as b:
                assert (b.info().grid_blocks == 0) == (bps == 0)
                b.step(steps)
                b.synchronize()
                out.append([(b.instance(k).get_f(), b.instance(k).force_history())
                            for k in range(len(cfgs))])
        for k in range(len(cfgs)):
            assert np.array_equal(out[0][k][0], out[1][k][0]), (th, k)
            assert np.array_equal(out[0][k][1], out[1][k][1]), (th, k)
            if ref_f is None:
                continue
            assert np.array_equal(out[0][k][0], ref_f[k]), (th, k)
        if ref_f is None:
            ref_f = [out[0][k][0] for k in range(len(cfgs))]
