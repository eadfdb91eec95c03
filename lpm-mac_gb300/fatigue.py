"""Cyclic fatigue loading.

``run_cycles`` is SolverFatigue::solveProblemCyclic (solver_fatigue.h:174-210)
run inside the library (lpm_fatigue_run): cycle N takes its loads f_min,
f_max, f_min from the spectrum at 2N, 2N+1, 2N+2 (the spectrum is held on the
device and the increments are formed there), each simulated cycle stands
for dN/dt real cycles (TimeMapMode Linear: int(1/tau); Exponential:
int(exp(t/tau)/tau) with t counting simulated cycles), and the run ends once
N reaches the spectrum's cycle count.  ``run_cycles_per_call`` drives the
same loop from Python with one lpm_fatigue_cycle call per cycle.
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


def run_cycles(lattice, bcs_unit, spectrum, n_interval, tau, mode=LINEAR, max_calls=None, **opts):
    """Runs the cyclic loading in the library; returns one record per
    simulated cycle (real cycle count N after it, dN/dt, iteration counts,
    new damage, mean strain energy, and a status: NOT_CONVERGED if a step of
    the cycle hit max_iter)."""
    from .capi import NOT_CONVERGED, OK, TIME_EXPONENTIAL, TIME_LINEAR
    st, recs = lattice.fatigue_run(bcs_unit, spectrum, n_interval, tau,
                                   TIME_LINEAR if mode == LINEAR else TIME_EXPONENTIAL,
                                   max_calls or 0, **opts)
    for r in recs:
        r["status"] = NOT_CONVERGED if r["unconverged_steps"] else OK
        r["new_damage"] = bool(r["new_damage"])
    return recs


def run_cycles_per_call(lattice, bcs_unit, spectrum, n_interval, tau, mode=LINEAR, max_calls=None, **opts):
    """The same loop driven from Python, one lpm_fatigue_cycle call per
    simulated cycle (the spectrum values passed from the host)."""
    n_cycles = 0.5 * (len(spectrum) - 1)
    N, t, out = 0, 0, []
    while N < n_cycles:
        f0, f1, f2 = spectrum[2 * N], spectrum[2 * N + 1], spectrum[2 * N + 2]
        jump = dNdt(tau, t, mode)
        t += 1
        r = lattice.fatigue_cycle(bcs_unit, f0, f1, f2, n_interval, jump, **opts)
        N += jump
        out.append(dict(N=N, dNdt=jump, **r))
        if max_calls is not None and len(out) >= max_calls:
            break
    return out
