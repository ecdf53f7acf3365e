"""Host logic of bench.py's extra legs, without a GPU: the sweep leg with
stand-ins for the batch (members, steps and the JSON it reports) and the
256 x 1024 plain-method leg with the FP64 oracle standing in for the device
library on a 2 cm run."""
import numpy as np


class _Member:
    def __init__(self):
        self.steps, self.z = 0, 0.0

    def stats(self):
        return {"steps": self.steps, "z": self.z}

    def analyze(self):
        return {"fluence": np.ones(4)}


class _Sweep:
    def __init__(self, params):
        self.params = params
        self.batch = type("B", (), {})()
        self.batch.members = [_Member() for _ in params]

    def tune(self, k):
        return {1: 2.0, 2: 1.5}

    def plan(self):
        return {"branches": 2, "dht_simt": [0] * len(self.params)}

    def run(self, zmax=None, nmax=0, z0=None):
        st = []
        for m in self.batch.members:
            m.steps += nmax
            m.z += 0.01 * nmax
            st.append({"steps": m.steps, "z": m.z, "status": 3})
        return 0, st

    def fields(self):
        return [np.full((2, 2), 1.0 + 1e-5, complex) for _ in self.params]

    def close(self):
        pass


class _Ref:
    def __init__(self, inp, precision=None, binding=None):
        h = _Member()
        h.set_option = lambda *a: None
        h.run = lambda z0, zmax, nmax: (1, {})
        h.get_field = lambda: np.ones((2, 2), complex)
        h.close = lambda: None
        self.handle = h

    def close(self):
        pass


def test_sweep_leg_reports_every_member(monkeypatch):
    import bench
    import filament_gb as fg
    from filament_gb import sweep
    monkeypatch.setattr(sweep, "Sweep", _Sweep)
    monkeypatch.setattr(fg, "Simulation", _Ref)
    r = bench.time_sweep(n=6, steps=4, warmup=1, oracle_members=3)
    assert "error" not in r, r.get("error")
    assert r["members"] == 6 and r["ranks"] == 1
    assert r["z_steps_total"] == 24 and r["status"] == [3] * 6
    assert r["tuner"]["branches"] == 2
    acc = r["accuracy_vs_fp64"]
    assert abs(acc["field_rel_l2_max"] - 1e-5) < 1e-9 and abs(acc["field_rel_l2_median"] - 1e-5) < 1e-9
    # the three cheapest members against the (stand-in) oracle
    oc = r["accuracy_vs_oracle"]
    assert len(oc["members"]) == 3 and abs(oc["field_rel_l2_max"] - 1e-5) < 1e-9
    costs = sorted(sweep.step_cost(p) for p in sweep.draw(6, 0))
    assert sorted(sweep.step_cost(dict(Nr=m["Nr"], Nt=m["Nt"])) for m in oc["members"]) == costs[:3]


def test_c1_leg_with_the_oracle_standing_in(monkeypatch, oracle_binding):
    import bench
    import filament_gb as fg
    prepare, Simulation = fg.prepare, fg.Simulation
    monkeypatch.setattr(fg, "prepare", lambda deck, **kw: dict(prepare(deck, **kw), zmax=0.02))
    monkeypatch.setattr(fg, "Simulation",
                        lambda inp, binding=None, precision="mixed": Simulation(inp, binding=oracle_binding,
                                                                               precision=precision))
    r = bench.time_c1(cpu_steps=3)
    for form in ("mixed", "fp64"):
        assert r[form]["steps"] == 20 and r[form]["status"] == 1
        assert abs(r[form]["z_end"] - 0.02) < 1e-12
    assert r["mixed"]["rel_l2_field_vs_fp64"] < 1e-12   # the oracle computes both forms in FP64
    assert r["cpu_oracle"]["steps"] == 3 and r["cpu_oracle"]["z_steps_per_s"] > 0


def test_accuracy_leg_with_the_oracle_standing_in(monkeypatch, oracle_binding):
    """accuracy_run's bookkeeping (every form against the oracle and
    against the GPU FP64 form) with the oracle standing in for the device
    library on a 2 cm run of a 64 x 512 grid."""
    import bench
    import filament_gb as fg
    prepare, Simulation = fg.prepare, fg.Simulation
    monkeypatch.setattr(bench, "WORKLOAD", dict(bench.WORKLOAD, Nr=64, Nt=512, rmax=2.0, tmin=-100.0, tmax=100.0))
    monkeypatch.setattr(fg, "Simulation",
                        lambda inp, binding=None, precision="mixed": Simulation(inp, binding=oracle_binding,
                                                                               precision=precision))
    r = bench.accuracy_run(0.02, 1000, zs=(0.01, 0.02))
    assert r["z_end"] == 0.02 and r["stops"] == [0.01, 0.02]
    for form in ("mixed", "mixed_simt", "fp64", "oracle"):
        assert abs(r[form]["z"] - 0.02) < 1e-12 and r[form]["steps"] >= 2
        assert [round(x["z"], 12) for x in r[form]["series"]] == [0.01, 0.02]
    for form in ("mixed", "mixed_simt"):
        assert r[form]["vs_oracle"]["field_rel_l2"] < 1e-12      # all FP64 here
        assert r[form]["vs_fp64_gpu"]["fluence_rel_l2"] < 1e-12
    assert r["fp64"]["vs_oracle"]["field_rel_l2"] < 1e-12


def test_reference_arm_prints_the_contract_line():
    """`bench.py --impl reference` times the FP64 oracle on the host threads
    (W untimed and K timed z-steps of the workload) and prints one JSON line
    with the arm's metric, the reference marker, its CPU baseline and an e2e
    block without device copies."""
    import json
    import os
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    out = subprocess.run([sys.executable, os.path.join(root, "bench.py"), "--impl", "reference",
                          "--steps", "2", "--warmup", "3"], capture_output=True, text=True, timeout=600,
                         cwd=root)
    assert out.returncode == 0, out.stderr[-2000:]
    line = json.loads(out.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["metric"] == "RT z-steps/s" and line["unit"] == "z-steps/s"
    assert line["steps"] == 2 and line["warmup"] == 3 and line["higher_is_better"] is True
    assert line["value"] > 0 and line["cpu_baseline"]["value"] == line["value"]
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["cores"] >= 1
    assert line["e2e"] == {"value": line["value"], "unit": "z-steps/s", "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}
    assert line["config"]["Nr"] == 1000 and line["config"]["Nt"] == 4096
