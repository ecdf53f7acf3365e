"""Batched parameter sweep of RT pulses on uneven grids.

The reference runs one deck per `Filament.run` call (src/Filament.jl:51-108);
a sweep there is a host loop over decks, each with its own field, model and
main loop.  Here the members of a sweep share one device and one CUDA graph
per z-step (`Batch`, fil_create_batch / fil_batch_run): every member keeps
its own grid, tables, field state and adaptive-dz controller, and the
autotuner (fil_batch_tune) picks each member's Hankel transform kernel and
the number of concurrent branches from measured step times.

`shard` splits the members over the ranks of a multi-GPU run (one process
per GPU, no data exchange; only the timing and the error maxima are
reduced).  `draw` makes the 64-pulse sweep's parameters from a seed: Nr from
{256, 512, 1000}, Nt from {1024, 2048, 4096}, peak power uniform in
2-10 Pcr, linear chirp (spectral phase phi2 (w - w0)^2 / 2) uniform in
+-500 fs^2, and beam radius w0 uniform in 0.5-2 mm, all with numpy's PCG64.
"""
import os

import numpy as np

from .backend import Batch
from .filament import Simulation
from .input import prepare

HERE = os.path.dirname(os.path.abspath(__file__))
RT_DECK = os.path.join(os.path.dirname(HERE), "decks", "filament_RT", "input.py")

NR_CHOICES = (256, 512, 1000)
NT_CHOICES = (1024, 2048, 4096)

# the members' common settings: the 1000 x 4096 filamentation workload's
# medium, window, integrator and step control
COMMON = dict(rmax=5.0, tmin=-200.0, tmax=200.0, ALG="RK4", dzphimax=0.1, dz_initial=1e-2, zmax=3.0)


def draw(n=64, seed=0):
    """Parameters of n sweep members: list of dicts (Nr, Nt, PPcr,
    chirp_fs2, beam_a0 in m)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    nr = rng.choice(NR_CHOICES, n)
    nt = rng.choice(NT_CHOICES, n)
    p = rng.uniform(2.0, 10.0, n)
    chirp = rng.uniform(-500.0, 500.0, n)
    w0 = rng.uniform(0.5, 2.0, n)
    return [dict(Nr=int(nr[i]), Nt=int(nt[i]), PPcr=float(p[i]), chirp_fs2=float(chirp[i]),
                 beam_a0=float(w0[i]) * 1e-3) for i in range(n)]


def step_cost(params):
    """Relative cost of one z-step of a member: the two Hankel GEMMs
    (Mpad^2 Nt, tensor cores) and the row work (Mpad Nt log Nt)."""
    mpad = (params["Nr"] + 127) // 128 * 128
    nt = params["Nt"]
    return 0.1 * mpad * mpad * nt + 40.0 * mpad * nt * np.log2(nt)


def shard(params, rank, world):
    """Indices of the members that rank `rank` of `world` runs: members are
    independent, so the sweep splits across GPUs without any exchange.
    Longest step first, each to the rank with the least total cost (ties
    to the lower rank); the same on every rank."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("bad rank %r of world %r" % (rank, world))
    order = sorted(range(len(params)), key=lambda i: (-step_cost(params[i]), i))
    load = [0.0] * world
    owner = [0] * len(params)
    for i in order:
        r = min(range(world), key=lambda k: (load[k], k))
        owner[i] = r
        load[r] += step_cost(params[i])
    return [i for i in range(len(params)) if owner[i] == rank]


def member_input(params, deck=RT_DECK, **over):
    """Input dict (Input.prepare) of one member."""
    kw = dict(COMMON)
    kw.update(params)
    kw.update(over)
    return prepare(deck, **kw)


class Sweep:
    """The members' simulations (host set-up, FP64) on one device batch.
    `sims[i].handle` is member i's handle; `batch` the fil_batch."""

    def __init__(self, params, precision="mixed", binding=None, deck=RT_DECK, **over):
        self.params = list(params)
        self.inputs = [member_input(p, deck, **over) for p in self.params]
        self.sims = [Simulation(inp, binding=binding, precision=precision, make_handle=False)
                     for inp in self.inputs]
        self.batch = Batch([s.problem for s in self.sims], binding)
        for s, h in zip(self.sims, self.batch.members):
            s.attach(h)

    def __len__(self):
        return len(self.sims)

    def tune(self, max_branches=16):
        return self.batch.tune(max_branches)

    def plan(self):
        return self.batch.plan()

    def run(self, zmax=None, nmax=10 ** 9, z0=None):
        """Every member from z0 (default: its current z) to zmax (default:
        the deck's), at most nmax steps."""
        n = len(self.sims)
        if z0 is None:
            z0 = []
            for s, m in zip(self.sims, self.batch.members):
                st = m.stats()
                z0.append(st["z"] if st["steps"] else s.z)
        if zmax is None:
            zmax = [s.zmax for s in self.sims]
        return self.batch.run(np.broadcast_to(np.asarray(z0, float), (n,)),
                              np.broadcast_to(np.asarray(zmax, float), (n,)), nmax)

    def fields(self):
        return [s.handle.get_field() for s in self.sims]

    def close(self):
        self.batch.close()
