"""Galactic code units of the reference (core/units.py:1-37): kpc, km/s,
1e10 Msun; time unit kpc/(km/s) ~= 0.978 Gyr."""

# Newton's constant in kpc (km/s)^2 / (1e10 Msun), core/units.py:21.
G = 43009.1725

KPC_PER_KM = 3.240779289e-17
GYR_PER_TIMEUNIT = 0.97781
MSUN_PER_MASSUNIT = 1.0e10

LENGTH_UNIT = "kpc"
VELOCITY_UNIT = "km/s"
MASS_UNIT = "1e10 Msun"
TIME_UNIT = "kpc/(km/s) ~= 0.978 Gyr"


def time_to_gyr(t: float) -> float:
    return t * GYR_PER_TIMEUNIT
