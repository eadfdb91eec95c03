"""Host side of the cyclic fatigue driver (fatigue.py), on the CPU: the
spectrum file format and the constant-amplitude spectrum of
SolverFatigue::readLoad (solver_fatigue.h:41-60), and the cycle jump of the
two TimeMapModes (solver_fatigue.h:174-210: Linear int(1/tau), Exponential
int(exp(t/tau)/tau))."""
import math

from lpm_cases import pkg

fat = pkg.fatigue


def test_constant_amplitude_spectrum():
    sp = fat.ca_spectrum(400.0, 0.1, 3)
    assert sp == [40.0, 400.0, 40.0, 400.0, 40.0, 400.0, 40.0]
    assert 0.5 * (len(sp) - 1) == 3  # cycles the driver reads from it


def test_read_spectrum_whitespace_separated(tmp_path):
    f = tmp_path / "load.txt"
    f.write_text("40\n400\n40 400\n\t40\n")
    assert fat.read_spectrum(str(f)) == [40.0, 400.0, 40.0, 400.0, 40.0]


def test_cycle_jump_of_both_time_maps():
    assert fat.dNdt(0.001, 0, fat.LINEAR) == 1000
    assert fat.dNdt(0.001, 17, fat.LINEAR) == 1000
    for t in range(6):
        assert fat.dNdt(0.5, t, fat.EXPONENTIAL) == int(1.0 / 0.5 * math.exp(t / 0.5))
    # the real cycle count after k simulated cycles of the linear map
    n, t = 0, 0
    for _ in range(3):
        n += fat.dNdt(0.001, t, fat.LINEAR)
        t += 1
    assert n == 3000
