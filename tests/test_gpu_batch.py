"""Batched sweep (fil_create_batch / fil_batch_tune / fil_batch_run) on the
GPU: members on uneven grids stepped by one CUDA graph per z-step must give
exactly the fields of the same problems run alone through fil_run (the same
kernels on the same data), and a member must agree with the FP64 oracle's
loop as a single handle does (relative L2 within 10x the mixed form's
one-step tolerance of 1e-5)."""
import numpy as np
import pytest

from gpu_helpers import rel_l2

pytestmark = pytest.mark.gpu

SMALL = dict(rmax=2.0, tmin=-100.0, tmax=100.0)

MEMBERS = [
    dict(Nr=64, Nt=512, PPcr=40.0, chirp_fs2=0.0, beam_a0=1.0e-3),
    dict(Nr=100, Nt=1024, PPcr=25.0, chirp_fs2=300.0, beam_a0=0.8e-3),
    dict(Nr=128, Nt=512, PPcr=60.0, chirp_fs2=-450.0, beam_a0=0.6e-3),
    dict(Nr=200, Nt=1024, PPcr=30.0, chirp_fs2=120.0, beam_a0=0.9e-3),
]


def _single(params, dht_simt, zmax, nmax):
    import filament_gb as fg
    from filament_gb import _abi, sweep
    sim = fg.Simulation(sweep.member_input(params, **SMALL))
    if dht_simt:
        sim.handle.set_option(_abi.OPT_DHT_SIMT, 1)
    code, st = sim.handle.run(0.0, zmax, nmax)
    E = sim.handle.get_field()
    sim.close()
    return code, st, E


def test_batch_members_match_single_runs(gpu_lib):
    from filament_gb import sweep
    sw = sweep.Sweep(MEMBERS, **SMALL)
    try:
        times = sw.tune(max_branches=4)
        assert set(times) <= {1, 2, 4} and all(t > 0 for t in times.values())
        plan = sw.plan()
        assert plan["branches"] in times
        assert len(plan["branch"]) == len(MEMBERS)
        assert all(0 <= b < plan["branches"] for b in plan["branch"])
        code, stats = sw.run(zmax=0.05, nmax=6, z0=0.0)
        assert code == 0
        fields = sw.fields()
    finally:
        sw.close()
    for i, p in enumerate(MEMBERS):
        c1, s1, E1 = _single(p, plan["dht_simt"][i], 0.05, 6)
        assert stats[i]["status"] == c1
        assert stats[i]["steps"] == s1["steps"]
        assert stats[i]["z"] == s1["z"]
        assert rel_l2(fields[i], E1) <= 1e-12, i


def test_batch_tune_restores_the_fields(gpu_lib):
    from filament_gb import sweep
    sw = sweep.Sweep(MEMBERS[:3], **SMALL)
    try:
        sw.run(zmax=1.0, nmax=2, z0=0.0)
        before = sw.fields()
        sw.tune(max_branches=2)
        after = sw.fields()
        for a, b in zip(after, before):
            assert np.array_equal(a, b)
    finally:
        sw.close()


def test_batch_members_stop_independently(gpu_lib):
    """Each member stops on its own zmax or Istop; the others go on."""
    from filament_gb import sweep
    sw = sweep.Sweep(MEMBERS[:3], **SMALL)
    try:
        zmax = [0.004, 0.02, 0.05]
        code, stats = sw.run(zmax=zmax, nmax=10 ** 6, z0=0.0)
        assert code == 0
        for st, zm in zip(stats, zmax):
            assert st["status"] == 1
            assert st["z"] >= zm and st["z"] - st["dz"] < zm
        assert stats[0]["steps"] < stats[2]["steps"]
        code, stats = sw.run(zmax=1.0, nmax=3, z0=0.0)
        assert [s["status"] for s in stats] == [3, 3, 3]
    finally:
        sw.close()


def test_batch_member_matches_oracle_loop(gpu_lib):
    import filament_gb as fg
    import oracle
    from filament_gb import _abi, sweep
    p = MEMBERS[1]
    sw = sweep.Sweep([MEMBERS[0], p], **SMALL)
    try:
        code, stats = sw.run(zmax=0.03, nmax=10 ** 6, z0=0.0)
        E = sw.fields()[1]
    finally:
        sw.close()
    r = fg.Simulation(sweep.member_input(p, **SMALL), binding=oracle.binding())
    code_r, st_r = r.handle.run(0.0, 0.03, 10 ** 6)
    assert code == 0 and code_r == 1 == stats[1]["status"]
    assert stats[1]["steps"] == st_r["steps"]
    assert stats[1]["z"] == pytest.approx(st_r["z"], rel=1e-5)
    assert rel_l2(E, r.handle.get_field()) < 1e-4


def test_every_member_matches_the_oracle_at_z_end(gpu_lib):
    """The sweep's per-member accuracy against the FP64 oracle of the
    reference's method (its loop: adaptive dz, plasma, RK4) at each
    member's own end of a 0.1 m run on the device controller, past the
    first adaptive-step reductions of the 25-60 Pcr members."""
    import filament_gb as fg
    import oracle
    from filament_gb import sweep
    sw = sweep.Sweep(MEMBERS, **SMALL)
    try:
        code, stats = sw.run(zmax=0.1, nmax=10 ** 6, z0=0.0)
        E = sw.fields()
    finally:
        sw.close()
    errs = []
    for i, p in enumerate(MEMBERS):
        r = fg.Simulation(sweep.member_input(p, **SMALL), binding=oracle.binding())
        code_r, st_r = r.handle.run(0.0, 0.1, 10 ** 6)
        assert code_r == 1 == stats[i]["status"] and stats[i]["steps"] == st_r["steps"]
        errs.append(rel_l2(E[i], r.handle.get_field()))
        r.close()
    print("per-member field error against the oracle at z = 0.1 m:", ["%.2e" % e for e in errs])
    assert max(errs) < 1e-4


def test_member_with_the_surrogate_matches_its_single_run(gpu_lib):
    """A member may arm the learned surrogate (its network kernels run on
    the member's own buffers inside the batch graph): its batch run equals
    the same problem armed and run alone, and the unarmed member equals its
    plain single run."""
    import filament_gb as fg
    from filament_gb import surrogate as S
    from filament_gb import sweep
    p0, p1 = MEMBERS[0], MEMBERS[1]
    net = S.Surrogate(p1["Nt"], seed=2)   # untrained: the g = 0 closed form
    zmax, nmax = 0.05, 30
    single = fg.Simulation(sweep.member_input(p1, **SMALL))
    net.arm(single.handle, every=5, tol=1.0)
    code_s, st_s = single.handle.run(0.0, zmax, nmax)
    E1 = single.handle.get_field()
    used_single = S.stats(single.handle)["steps_used"]
    single.close()
    _, _, E0 = _single(p0, False, zmax, nmax)
    sw = sweep.Sweep([p0, p1], **SMALL)
    try:
        net.arm(sw.batch.members[1], every=5, tol=1.0)
        code, stats = sw.run(zmax=zmax, nmax=nmax, z0=0.0)
        E = sw.fields()
        used = S.stats(sw.batch.members[1])["steps_used"]
    finally:
        sw.close()
    net.close()
    assert used == used_single > 0
    assert stats[1]["steps"] == st_s["steps"]
    assert rel_l2(E[1], E1) < 1e-12 and rel_l2(E[0], E0) < 1e-12
