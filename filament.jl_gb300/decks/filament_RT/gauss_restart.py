# Initial condition that continues a stopped run from a saved field, the
# counterpart of the reference's examples/RT/gauss_restart.jl.  The run wrote
# its field snapshots as <prefix>plot_field_NNN.npy (Re(E) on the same grid)
# with their z values (in zu) in <prefix>plot_fields_z.npy; this file takes
# snapshot `restart_index` from `restart_dir` (both overridable, e.g.
# prepare(deck, file_initial_condition="gauss_restart.py",
# restart_dir=".../results", restart_index=2)).  The real field becomes the
# analytic signal on upload, as a fresh initial condition does.
import os

restart_dir = globals().get("restart_dir", os.path.join(DECKDIR, "results"))
restart_index = globals().get("restart_index", 1)

lam0 = 0.8e-6
z = float(np.load(os.path.join(restart_dir, "plot_fields_z.npy"))[restart_index - 1]) * zu


def initial_condition(r, t, ru, tu, Iu):
    E = np.load(os.path.join(restart_dir, "plot_field_%03d.npy" % restart_index))
    if E.shape != (len(r), len(t)):
        raise ValueError("the saved field is on another grid")
    return E.astype(np.complex128)
