"""Factor-level agreement of a GPU epoch with the FP64 oracle's epoch.

For each mode m, with F0 the factors before the epoch, R the oracle's factors
after it and F the GPU's:
  deviation  ||F - R|| / ||R - F0||        (0 = identical, 1 = no movement)
  slope      <F - F0, R - F0> / ||R - F0||^2   (1 = same movement, 0 = none,
             0.5 = half the step); zero-mean rounding noise does not bias it
A kernel that skips updates, applies part of each, or updates the wrong rows
fails both; an epoch at half the learning rate has slope ~0.5.
"""
import numpy as np

# FP32/FP64 timed paths: measured deviation <= 0.044, slope 1.002-1.039
DEV_TOL = 0.1
SLOPE_TOL = 0.08
# BF16: slope measured 0.93-1.05; residual in BF16 ulps of the oracle value
BF16_SLOPE_TOL = 0.15
BF16_ULP_RMS = 3.0


def agreement(F, R, F0):
    """[(deviation, slope)] per mode."""
    out = []
    for f, r, f0 in zip(F, R, F0):
        mv = r - f0
        n2 = float((mv * mv).sum())
        if n2 == 0.0:
            out.append((float("inf"), 0.0))
            continue
        d = f - r
        out.append((float(np.sqrt((d * d).sum() / n2)), float(((f - f0) * mv).sum() / n2)))
    return out


def bf16_ulp_residual(F, R):
    """RMS of (F - R) over every element, in units of one BF16 ulp (8
    significant bits) of each mode's RMS value (elements near zero have
    far smaller ulps than the rows' typical ones, so a per-element ulp would
    let them dominate)."""
    tot, cnt = 0.0, 0
    for f, r in zip(F, R):
        rms = max(float(np.sqrt((r * r).mean())), 2.0 ** -30)
        _, e = np.frexp(rms)  # rms = m 2^e, m in [0.5, 1): ulp = 2^(e - 8)
        q = (f - r) / np.ldexp(1.0, e - 8)
        tot += float((q * q).sum())
        cnt += q.size
    return float(np.sqrt(tot / max(cnt, 1)))


def check_fp(F, R, F0, dev_tol=DEV_TOL, slope_tol=SLOPE_TOL):
    ag = agreement(F, R, F0)
    for m, (dev, slope) in enumerate(ag):
        if not (dev <= dev_tol and abs(slope - 1.0) <= slope_tol):
            return False, "mode %d: deviation %.4g slope %.4g (all modes %s)" % (m, dev, slope, ag)
    return True, ""


def check_bf16(F, R, F0, slope_tol=BF16_SLOPE_TOL, ulp_rms=BF16_ULP_RMS):
    ag = agreement(F, R, F0)
    for m, (dev, slope) in enumerate(ag):
        if abs(slope - 1.0) > slope_tol:
            return False, "mode %d: slope %.4g (all modes %s)" % (m, slope, ag)
    u = bf16_ulp_residual(F, R)
    if u > ulp_rms:
        return False, "residual %.3g BF16 ulps RMS (modes %s)" % (u, ag)
    return True, ""
