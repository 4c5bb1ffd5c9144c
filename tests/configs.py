"""Seeded configurations of the benchmark spec, made with the oracle (whose
pure-gauge HMC and RNG are pinned bit for bit to the reference's own
HMCPureGauge / ParallelRng2 in tests/golden/gauge_ref.json)."""
import numpy as np

from oracle import oracle as O


def reference_thermalised_links(g, beta: float, seed: int, ntraj: int, compact: bool = True, nsteps: int = 40,
                                n_noreject: int = 10):
    """The reference pure-gauge driver's recipe (src/both/gauge.cu:127-130,
    466-492): ParallelRng2(seed); U.gaussian(rng, 0.2); one momentum draw
    (pi.gaussian before the HMC is built); n_noreject trajectories accepted
    unconditionally, then ntraj Metropolis trajectories of tmax = 1, nsteps
    leapfrog steps, with the reference's force (theta, also for the compact
    action).  Returns (links, acceptance of the ntraj trajectories)."""
    rng = O.Rng(g, seed)
    A = np.ascontiguousarray(rng.gaussian_links(0.2))
    rng.gaussian_links(1.0)
    for _ in range(n_noreject):
        O.hmc_pure_gauge(g, rng, A, beta, compact, False, 1.0, nsteps, no_reject=True)
    acc = 0
    for _ in range(ntraj):
        a, _ = O.hmc_pure_gauge(g, rng, A, beta, compact, False, 1.0, nsteps)
        acc += int(a)
    return A, acc / max(1, ntraj)
