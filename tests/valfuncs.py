"""Time-dependent boundary values and body force of the VAL_FUNC golden
cases, as Python callbacks f(t, x, y, z).

The same expressions, in the same order of operations, are compiled into
the reference driver that produced the fixtures (oracle/ref_driver.c), so
the GPU path samples the same doubles the reference evaluated: only +, -
and * appear, which round identically on every IEEE host.
"""


def pulse_u(t, x, y, z):
    return (1.0 + 3.0 * t) * (1.0 - 0.2 * y * y) * (1.0 - 0.25 * z * z)


def pulse_v(t, x, y, z):
    return 0.2 * t * z


def pulse_w(t, x, y, z):
    return -0.1 * t * y + 0.05 * x


def ramp_p(t, x, y, z):
    return 0.5 * t + 0.1 * y - 0.05 * z * t


def swirl_f1(t, x, y, z):
    return 0.02 * (1.0 + t) * y


def swirl_f2(t, x, y, z):
    return -0.03 * x * t + 0.01 * z


def swirl_f3(t, x, y, z):
    return 0.01 * (x - y) * t


BC_FUNCS = {"pulse": (pulse_u, pulse_v, pulse_w), "ramp": (ramp_p,)}
FORCE_FUNCS = {"swirl": (swirl_f1, swirl_f2, swirl_f3)}
