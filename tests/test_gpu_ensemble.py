"""The batched ensemble: members with uneven grids and parameters stepped
together through one captured CUDA graph.  Each member must match, bit for
bit, the same instance run alone through the single-instance path (FP64 and
the split form); tuning changes tile shapes only, never results.  Also the
graph replay of the single-instance step against eager launches."""
import numpy as np
import pytest

from fug30v0kxc_gb300.params import VEC_PREC_FP64, VEC_PREC_SPLIT, convection_params
from fug30v0kxc_gb300.solver import P3D, Ensemble

pytestmark = pytest.mark.gpu

FIELDS = ("r", "t", "u", "v", "w", "pol", "tor", "bx", "by", "bz")


def members():
    a = convection_params(64, 64, 33, ra=3e4, q=100.0, eta_contrast=5.0, precision=VEC_PREC_SPLIT)
    b = convection_params(32, 32, 17, ra=1e5, q=0.0, eta_contrast=1.0, precision=VEC_PREC_SPLIT)
    c = convection_params(48, 48, 21, ra=5e5, q=1000.0, eta_contrast=20.0, precision=VEC_PREC_SPLIT)
    d = convection_params(64, 32, 25, ra=1e5, q=100.0, eta_contrast=5.0, precision=VEC_PREC_FP64)
    for i, p in enumerate((a, b, c, d)):
        p.seed_base = 1996 + 7 * i
        p.ndu06 = 15
    return [a, b, c, d]


@pytest.mark.parametrize("tune", [False, True])
def test_members_match_single_instance(tune, tmp_path):
    ps = members()
    ens = Ensemble(ps)
    ens.start()
    if tune:
        cache = str(tmp_path / "tune.txt")
        ens.tune(steps=2, cache=cache)
        lines = open(cache).read().split("\n")
        assert len([l for l in lines if l.strip()]) == 4
    assert ens.step(25) == 0
    ens.sync()
    for p, m in zip(ps, ens.members):
        solo = P3D(p)
        solo.start()
        assert solo.step(25) == 0
        for n in FIELDS:
            assert np.array_equal(m.get(n), solo.get(n)), (n, p.nx, p.ny, p.nz)
        assert m.scalars().dt == solo.scalars().dt
        solo.close()
    ens.close()


def batch_members(n, nx, ny, nz):
    """n members of one grid: magnetic (Q 100, 1000) and non-magnetic ones,
    uneven Ra and eta contrast, a distinct noise seed each."""
    qs, etas, ras = (0.0, 100.0, 1000.0), (1.0, 5.0, 20.0), (2e4, 1e5, 5e5, 1e6)
    ps = []
    for i in range(n):
        p = convection_params(nx, ny, nz, ra=ras[i % 4], q=qs[i % 3], eta_contrast=etas[(i // 3) % 3],
                              precision=VEC_PREC_SPLIT)
        p.seed_base = 2024 + 11 * i
        p.ndu06 = 1000000
        ps.append(p)
    return ps


def test_batched_members_match_single_instance():
    """18 members of one grid: two batches (at most 16 members per launch),
    80 jobs in a hydro line launch, magnetic and non-magnetic members in one
    batch (the first one non-magnetic); 25 steps cover the calcdt and
    dealias steps.  Fewer than 30 launches per batch and step; every member
    bit-identical to its solo run."""
    ps = batch_members(18, 32, 32, 17)
    ens = Ensemble(ps)
    ens.start()
    assert ens.step(5) == 0
    ens.sync()
    # graph replays: one launch per kernel for each batch (two batches here),
    # not one per member
    l0 = sum(m.launch_count() for m in ens.members)
    assert ens.step(10) == 0
    ens.sync()
    per_step = (sum(m.launch_count() for m in ens.members) - l0) / 10
    assert per_step < 2 * 30, per_step
    assert ens.step(10) == 0
    ens.sync()
    for p, m in zip(ps, ens.members):
        solo = P3D(p)
        solo.start()
        assert solo.step(25) == 0
        for n in FIELDS:
            assert np.array_equal(m.get(n), solo.get(n)), (n, p.chand, p.eta_contrast)
        assert m.scalars().dt == solo.scalars().dt
        solo.close()
    ens.close()


def test_graph_replay_matches_eager():
    p = convection_params(64, 64, 33, eta_contrast=20.0, precision=VEC_PREC_SPLIT)
    p.ndu06 = 7
    a, b = P3D(p), P3D(p)
    b.use_graphs(False)
    a.start(); b.start()
    assert a.step(23) == 0 and b.step(23) == 0
    for n in FIELDS:
        assert np.array_equal(a.get(n), b.get(n)), n
    assert a.launch_count() == b.launch_count()
