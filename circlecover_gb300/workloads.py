"""Seeded synthetic workloads for the prover, bit-identical on every IEEE-754
platform.

The random source is a counter-based splitmix64 on uint64 (wrapping integer
arithmetic), and the only non-elementary function needed, 2**x, is a
fixed-order Taylor polynomial; numpy's +, -, *, / and sqrt are correctly
rounded.  So x86 and Arm hosts generate the same boxes from the same seed and
no fixture of random inputs has to be stored.
"""
import math

import numpy as np

TIGHT_BOX = np.dtype([("la", "<f8", (2,)), ("r", "<f8", (4, 2))])
SB_BOX = np.dtype([("la", "<f8", (2,)), ("r", "<f8", (6, 2))])

# sqrt(sqrt(7)/2 - 1/4): aspect ratio where the 2-disk worst case takes over
LAMBDA_2 = math.sqrt(math.sqrt(7.0) / 2.0 - 0.25)
TIGHT_LAMBDA_MAX = 2.0898841580413818342
DBL_MAX = np.finfo(np.float64).max

_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)
_GOLD = np.uint64(0x9E3779B97F4A7C15)


def _mix(x):
    with np.errstate(over="ignore"):
        x = x ^ (x >> np.uint64(30))
        x = x * _M1
        x = x ^ (x >> np.uint64(27))
        x = x * _M2
        x = x ^ (x >> np.uint64(31))
    return x


def uniform(seed, index, stream):
    """U[0,1) doubles for a counter range; `index` is a uint64 array."""
    with np.errstate(over="ignore"):
        key = _mix(np.uint64(seed) * _GOLD + np.uint64(stream) * np.uint64(0xD1B54A32D192ED03))
        x = _mix(index.astype(np.uint64) * _GOLD + key)
    return (x >> np.uint64(11)).astype(np.float64) * (2.0 ** -53)


_LN2 = 0.6931471805599453
_EXP2_COEF = []
_c = 1.0
for _k in range(18):
    _EXP2_COEF.append(_c)
    _c = _c * _LN2 / (_k + 1)


def exp2(t):
    """2**t with a fixed evaluation order (deterministic across platforms)."""
    t = np.asarray(t, dtype=np.float64)
    k = np.floor(t)
    f = t - k
    p = np.full_like(f, _EXP2_COEF[-1])
    for c in reversed(_EXP2_COEF[:-1]):
        p = p * f + c
    return np.ldexp(p, k.astype(np.int32))


def critical_weight_point(lam):
    """Point value of the critical total weight critical_ratio(la) * la
    (reference: tight_rectangle/critical_ratio.cu:58-86), round-to-nearest;
    used only to place synthetic boxes near the critical amount."""
    lam = np.asarray(lam, dtype=np.float64)
    l2 = lam * lam
    three = (3.0 / 256.0) * (16.0 * l2 + 40.0 + 9.0 / l2)
    two = 0.25 * l2 + 0.5
    return np.where(lam <= LAMBDA_2, three, two)


def tight_microbench(n, seed=1, start=0, eps_lo=1e-6, eps_hi=1e-1):
    """Boxes of the batched-criteria microbench (2**24 boxes at full size):

    * lambda ~ U[1,4];
    * r1 ~ U[0.02,1]*sqrt(lambda), r2 = u*r1, r3 = v*r2 with u, v ~ U(0,1];
      the boxes hold weights w_i = r_i**2;
    * every interval is [c - d/2, c + d/2] around its point value with d
      log-uniform in [2**-20, 2**-4]; lower bounds clamped at 0 (lambda at 1);
    * total weight = critical_weight(lambda) * (1 + eps), eps log-uniform in
      [eps_lo, eps_hi]; R = total - w1 - w2 - w3 and r4**2 = [0, min(w3.ub, R)].

    `start` offsets the counter, so any slice of the full set can be made alone.
    """
    idx = np.arange(start, start + n, dtype=np.uint64)
    u = [uniform(seed, idx, s) for s in range(10)]
    lam = 1.0 + 3.0 * u[0]
    r1 = (0.02 + 0.98 * u[1]) * np.sqrt(lam)
    r2 = (1.0 - u[2]) * r1
    r3 = (1.0 - u[3]) * r2
    w = [r1 * r1, r2 * r2, r3 * r3]
    widths = [exp2(-20.0 + 16.0 * u[4 + k]) for k in range(4)]
    log2_10 = 3.321928094887362
    l_lo, l_hi = math.log10(eps_lo), math.log10(eps_hi)
    eps = exp2((l_lo + (l_hi - l_lo) * u[8]) * log2_10)

    out = np.zeros(n, dtype=TIGHT_BOX)
    out["la"][:, 0] = np.maximum(1.0, lam - 0.5 * widths[0])
    out["la"][:, 1] = lam + 0.5 * widths[0]
    for k in range(3):
        out["r"][:, k, 0] = np.maximum(0.0, w[k] - 0.5 * widths[k + 1])
        out["r"][:, k, 1] = w[k] + 0.5 * widths[k + 1]
    total = critical_weight_point(lam) * (1.0 + eps)
    R = total - w[0] - w[1] - w[2]
    out["r"][:, 3, 0] = 0.0
    out["r"][:, 3, 1] = np.minimum(out["r"][:, 2, 1], R)
    return out


def tight_near_critical(n, seed=5, start=0, frac_near=0.9):
    """Near-critical stress boxes: a fraction `frac_near` has total weight
    within 1e-4 (relative) of the critical weight (eps ~ U[-1e-4, 1e-4]); the
    rest are drawn like tight_microbench."""
    base = tight_microbench(n, seed=seed, start=start)
    idx = np.arange(start, start + n, dtype=np.uint64)
    pick = uniform(seed, idx, 20) < frac_near
    lam = 0.5 * (base["la"][:, 0] + base["la"][:, 1])
    eps = (2.0 * uniform(seed, idx, 21) - 1.0) * 1e-4
    wc = [0.5 * (base["r"][:, k, 0] + base["r"][:, k, 1]) for k in range(3)]
    R = critical_weight_point(lam) * (1.0 + eps) - wc[0] - wc[1] - wc[2]
    base["r"][:, 3, 1] = np.where(pick, np.minimum(base["r"][:, 2, 1], R), base["r"][:, 3, 1])
    return base


SB_UB_DISK_WEIGHT = 9.0 / 64.0
SB_CRITICAL_RATIO = 0.61


def sb_boxes(n, seed=3, start=0, la_lo=1.0, la_hi=2.5, heavy=0.7):
    """Boxes of the size-bound proof: lambda ~ U[la_lo, la_hi]; six weights
    r1 >= ... >= r6 <= 9/64.  A fraction `heavy` of the boxes has large
    disks (each weight u * 9/64 with u^(1/4), u ~ U(0,1], so most are close
    to the bound) and a remaining weight R = 0.61 lambda - sum near 0, where
    the expensive strategies are reached; the rest has uniform weights.
    Interval widths log-uniform in [2**-20, 2**-6]; lower bounds >= 0."""
    idx = np.arange(start, start + n, dtype=np.uint64)
    lam = la_lo + (la_hi - la_lo) * uniform(seed, idx, 0)
    pick = uniform(seed, idx, 1) < heavy
    w = []
    for k in range(6):
        u = 1.0 - uniform(seed, idx, 2 + k)
        heavy_w = np.sqrt(np.sqrt(u)) * SB_UB_DISK_WEIGHT
        w.append(np.where(pick, heavy_w, u * SB_UB_DISK_WEIGHT))
    w = -np.sort(-np.stack(w), axis=0)  # descending per box
    out = np.zeros(n, dtype=SB_BOX)
    wl = exp2(-20.0 + 14.0 * uniform(seed, idx, 8))
    out["la"][:, 0] = np.maximum(1.0, lam - 0.5 * wl)
    out["la"][:, 1] = lam + 0.5 * wl
    for k in range(6):
        wk = exp2(-20.0 + 14.0 * uniform(seed, idx, 9 + k))
        out["r"][:, k, 0] = np.maximum(0.0, w[k] - 0.5 * wk)
        out["r"][:, k, 1] = np.minimum(SB_UB_DISK_WEIGHT, w[k] + 0.5 * wk)
    # scale heavy boxes so that the six disks nearly exhaust 0.61 lambda
    total = SB_CRITICAL_RATIO * lam
    s = w.sum(axis=0)
    scale = np.where(pick & (s > total), total / s * (1.0 - 1e-3 * uniform(seed, idx, 16)), 1.0)
    out["r"] *= scale[:, None, None]
    return out


def sb_root(la_lo=1.0, la_hi=2.5):
    """Root box of the size-bound proof (rectangle_size_bound.cu:317-320)."""
    b = np.zeros(1, dtype=SB_BOX)
    b["la"][0] = (la_lo, la_hi)
    for k in range(6):
        b["r"][0, k] = (0.0, SB_UB_DISK_WEIGHT)
    return b[0]


def tight_root(la_lo=1.0, la_hi=TIGHT_LAMBDA_MAX):
    """Root box of the tight proof (reference: tight_rectangle.cu:461-464)."""
    b = np.zeros(1, dtype=TIGHT_BOX)
    b["la"][0] = (la_lo, la_hi)
    for k in range(4):
        b["r"][0, k] = (0.0, DBL_MAX)
    return b[0]


def to_soa(boxes):
    """AoS boxes -> (10, n) float64 array: la.lb, la.ub, r1.lb, r1.ub, ..."""
    n = len(boxes)
    flat = boxes.view(np.float64).reshape(n, -1)
    return np.ascontiguousarray(flat.T)
