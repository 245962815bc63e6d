"""Post-processing of the running statistics (f8_stats_begin / f8_stats_read)
in the reference's forms: the time average and its z average (ave_mean,
fenep_mpi.f90:2010-2033) and the temporal power spectrum of the centre-line
probes (power_spectrum, fenep_mpi.f90:2799-2862)."""
from __future__ import annotations

import numpy as np


def time_mean(sums, nsteps: int):
    """U_ave = sum / Nstep for the three components."""
    return tuple(s / nsteps for s in sums)


def ave_mean(mean):
    """z average of each mean field, broadcast back over z (ave_mean); arrays
    are (NZ, NY, NX)."""
    return tuple(np.broadcast_to(m.mean(axis=0), m.shape).copy() for m in mean)


def power_spectrum(probes):
    """(3, Nstep/2 + 1): for each component, sum over k of |u_hat(k, f)|^2 / 2
    with u_hat the real-to-complex transform of the probe series over the
    Nstep steps divided by Nstep (probes: (3, Nstep, NZ))."""
    n = probes.shape[1]
    hat = np.fft.rfft(probes, axis=1) / n
    return np.sum(np.abs(hat) ** 2, axis=2) / 2.0
