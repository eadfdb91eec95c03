"""Cyclic fatigue loading over lpm_fatigue_cycle.

``run_cycles`` follows SolverFatigue::solveProblemCyclic
(solver_fatigue.h:174-210): cycle N takes its loads f_min, f_max, f_min from
the spectrum at 2N, 2N+1, 2N+2, each simulated cycle stands for dN/dt real
cycles (TimeMapMode Linear: int(1/tau); Exponential: int(exp(t/tau)/tau)
with t counting simulated cycles), and the run ends once N reaches the
spectrum's cycle count.  Every cycle is one library call, so the load steps,
Newton solves, state updates and the fatigue damage update of a cycle run
back to back on the device.
"""
import math

LINEAR, EXPONENTIAL = "linear", "exponential"


def read_spectrum(path):
    """Load spectrum file: whitespace-separated values, f_min first, then
    f_max, f_min, ... (SolverFatigue::readLoad, solver_fatigue.h:41-60)."""
    with open(path) as f:
        return [float(v) for v in f.read().split()]


def ca_spectrum(f_max, R, ncycles):
    """Constant-amplitude spectrum f_min, f_max, f_min, ... for ncycles."""
    f_min = R * f_max
    return [f_min] + [f_max, f_min] * ncycles


def dNdt(tau, t, mode=LINEAR):
    if mode == LINEAR:
        return int(1.0 / tau)
    return int(1.0 / tau * math.exp(t / tau))


def run_cycles(lattice, bcs_unit, spectrum, n_interval, tau, mode=LINEAR, max_calls=None, on_cycle=None, **opts):
    """Runs the cyclic loading; returns one record per simulated cycle
    (real cycle count N after it, dN/dt, and the call's result)."""
    n_cycles = 0.5 * (len(spectrum) - 1)
    N, t, out = 0, 0, []
    while N < n_cycles:
        f0, f1, f2 = spectrum[2 * N], spectrum[2 * N + 1], spectrum[2 * N + 2]
        jump = dNdt(tau, t, mode)
        t += 1
        r = lattice.fatigue_cycle(bcs_unit, f0, f1, f2, n_interval, jump, **opts)
        N += jump
        out.append(dict(N=N, dNdt=jump, **r))
        if on_cycle:
            on_cycle(N, r)
        if max_calls is not None and len(out) >= max_calls:
            break
    return out
