"""Action-potential markers, computed identically for oracle and GPU traces.

The reference has no APD or upstroke implementation on the electrophysiology side, so
the definitions are fixed here:

* upstroke time: first upward crossing of -20 mV at or after the beat's stimulus time,
  linearly interpolated between samples;
* APD90: time from the upstroke to the first downward crossing, after the beat's peak,
  of V90 = Vpeak - 0.9 * (Vpeak - Vrest), Vrest being the sample at the stimulus time;
  linearly interpolated.

Traces are (n_cells, n_samples) in volts, sampled every `dt_sample` seconds from t0.
"""
from __future__ import annotations

import numpy as np


def _first_cross(v: np.ndarray, level: np.ndarray, start: np.ndarray, up: bool):
    """Index i (>= start) of the first sample pair (i, i+1) crossing level; -1 if none."""
    n, m = v.shape
    idx = np.arange(m - 1)[None, :]
    a, b = v[:, :-1], v[:, 1:]
    lv = level[:, None]
    hit = (a < lv) & (b >= lv) if up else (a > lv) & (b <= lv)
    hit &= idx >= start[:, None]
    any_hit = hit.any(axis=1)
    first = np.where(any_hit, hit.argmax(axis=1), -1)
    return first


def _interp(v, i, level):
    rows = np.arange(v.shape[0])
    a = v[rows, i]
    b = v[rows, i + 1]
    frac = np.where(b != a, (level - a) / np.where(b != a, b - a, 1.0), 0.0)
    return i + frac


def ap_markers(trace: np.ndarray, dt_sample: float, t_stim: float, t_end: float | None = None,
               t0: float = 0.0, level_up: float = -0.020):
    """Upstroke time and APD90 [s] for the beat stimulated at t_stim (window up to t_end).

    Returns (t_up, apd90, vpeak); NaN where a marker does not exist in the window.
    """
    v = np.asarray(trace, np.float64)
    if v.ndim == 1:
        v = v[None, :]
    n, m = v.shape
    s0 = int(np.floor((t_stim - t0) / dt_sample + 1e-9))
    s1 = m if t_end is None else min(m, int(np.floor((t_end - t0) / dt_sample + 1e-9)) + 1)
    s0 = max(0, min(s0, m - 2))
    w = v[:, :s1]
    vrest = w[:, s0]
    start = np.full(n, s0)
    iu = _first_cross(w, np.full(n, level_up), start, up=True)
    ok = iu >= 0
    t_up = np.full(n, np.nan)
    apd = np.full(n, np.nan)
    vpeak = np.full(n, np.nan)
    if ok.any():
        fu = _interp(w[ok], iu[ok], level_up)
        t_up[ok] = t0 + fu * dt_sample
        seg = w[ok].copy()
        cols = np.arange(s1)[None, :]
        seg = np.where(cols >= iu[ok][:, None], seg, -np.inf)
        ipk = seg.argmax(axis=1)
        vp = w[ok][np.arange(ok.sum()), ipk]
        vpeak[ok] = vp
        v90 = vp - 0.9 * (vp - vrest[ok])
        ir = _first_cross(w[ok], v90, ipk, up=False)
        ok2 = ir >= 0
        fr = np.full(ok.sum(), np.nan)
        if ok2.any():
            fr[ok2] = _interp(w[ok][ok2], ir[ok2], v90[ok2])
        apd[ok] = (fr - fu) * dt_sample
    return t_up, apd, vpeak


def beat_markers(trace, dt_sample, t_stims, t0=0.0):
    """ap_markers for each beat; t_stims is a list of stimulus times (per beat) or an
    array (n_beats, n_cells) of per-cell stimulus times. Returns arrays (n_beats, n_cells)."""
    v = np.asarray(trace, np.float64)
    n = v.shape[0]
    ts = np.asarray(t_stims, np.float64)
    if ts.ndim == 1:
        ts = np.repeat(ts[:, None], n, axis=1)
    out_up, out_apd = [], []
    for b in range(ts.shape[0]):
        ups = np.full(n, np.nan)
        apds = np.full(n, np.nan)
        # group cells by identical window to keep it vectorised
        for t_s in np.unique(ts[b]):
            sel = ts[b] == t_s
            nxt = ts[b + 1][sel].min() if b + 1 < ts.shape[0] else None
            u, a, _ = ap_markers(v[sel], dt_sample, t_s, nxt, t0)
            ups[sel] = u
            apds[sel] = a
        out_up.append(ups)
        out_apd.append(apds)
    return np.array(out_up), np.array(out_apd)
