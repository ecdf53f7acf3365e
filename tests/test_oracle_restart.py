"""Restart from a saved field (the reference's examples/RT/gauss_restart.jl):
a run writes its field snapshots (plot_field_NNN.npy, Re(E), with their z
in plot_fields_z.npy, the content of plot.h5's field group); the deck's
gauss_restart.py takes one back as the initial condition at its z, and the
continued run ends at the uninterrupted run's field.  From the first
snapshot (z = 0) the two runs are the same run; from a later one they
differ only by the negative-frequency part of the field that the real
snapshot drops (6e-8 here).  Run on the oracle, the ABI's CPU twin."""
import os

import numpy as np
import pytest

from gpu_helpers import FIL_DECK

KW = dict(Nr=64, Nt=512, rmax=2.0, tmin=-100.0, tmax=100.0, zmax=0.01, dz_plothdf=0.005)


@pytest.mark.parametrize("index, tol", [(1, 1e-14), (2, 1e-6)])
def test_restart_from_a_saved_field(oracle_binding, tmp_path, index, tol):
    import filament_gb as fg
    run = fg.run(fg.prepare(FIL_DECK, **KW), binding=oracle_binding, write_files=True, outdir=str(tmp_path))
    E_run = run.handle.get_field()
    res = os.path.join(str(tmp_path), "results")
    zs = np.load(os.path.join(res, "plot_fields_z.npy"))
    assert np.allclose(zs, [0.0, 0.005, 0.01])
    inp = fg.prepare(FIL_DECK, file_initial_condition="gauss_restart.py", restart_dir=res,
                     restart_index=index, **KW)
    assert inp["z"] == zs[index - 1]
    cont = fg.run(inp, binding=oracle_binding, write_files=False)
    assert cont.z == pytest.approx(run.z, rel=1e-12)
    E = cont.handle.get_field()
    assert np.linalg.norm(E - E_run) <= tol * np.linalg.norm(E_run)
    run.close()
    cont.close()
