"""Terrain statistics shared by the statistical parity checks of the
parallel mode against the reference's sequential World::erode
(source/world.hpp:36-77).

- quantile profile: the sorted heights averaged over equal-count bins; the
  mean absolute difference of two profiles is the 1-Wasserstein distance of
  the two height histograms at that resolution (exact when every bin holds
  one value);
- log radial spectrum: log10 of the radially averaged power spectrum of the
  mean-free height map in 32 wavenumber bins up to Nyquist (ripple and dune
  wavelengths);
- the mean height (sediment carried off the map).
"""
from __future__ import annotations

import numpy as np

PROFILE_BINS = 4096
SPECTRUM_BINS = 32


def quantile_profile(a, bins: int = PROFILE_BINS) -> np.ndarray:
    s = np.sort(np.asarray(a, np.float64).ravel())
    if s.size % bins:
        raise ValueError(f"{s.size} heights do not split into {bins} equal bins")
    return s.reshape(bins, -1).mean(axis=1)


def w1(a, b) -> float:
    """1-Wasserstein distance between the height histograms of two maps."""
    return float(np.mean(np.abs(np.sort(np.ravel(a)).astype(np.float64) - np.sort(np.ravel(b)))))


def w1_profiles(pa, pb) -> float:
    return float(np.mean(np.abs(np.asarray(pa, np.float64) - np.asarray(pb, np.float64))))


def log_spectrum(a) -> np.ndarray:
    a = np.asarray(a, np.float64)
    f = np.abs(np.fft.rfft2(a - a.mean())) ** 2
    ky = np.fft.fftfreq(a.shape[0])[:, None]
    kx = np.fft.rfftfreq(a.shape[1])[None, :]
    k = np.sqrt(kx ** 2 + ky ** 2)
    edges = np.linspace(0, 0.5, SPECTRUM_BINS + 1)
    idx = np.digitize(k.ravel(), edges)
    s = np.array([f.ravel()[idx == i].mean() if np.any(idx == i) else 0.0
                  for i in range(1, SPECTRUM_BINS + 1)])
    return np.log10(s + 1e-12)


def spec_dist_logs(la, lb) -> float:
    return float(np.sqrt(np.mean((np.asarray(la) - np.asarray(lb)) ** 2)))


def spec_dist(a, b) -> float:
    """RMS distance between the log radial spectra of two maps."""
    return spec_dist_logs(log_spectrum(a), log_spectrum(b))


def summary(a) -> dict:
    a = np.asarray(a)
    return {"profile": quantile_profile(a), "logspec": log_spectrum(a), "mean": float(np.mean(a, dtype=np.float64))}
