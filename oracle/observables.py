"""FP64 host oracle of the ensemble observables (test infrastructure only).

The GPU reduces these in double precision (sc_observe, sc_pair_histogram in
spatial_cell_gb300/csrc/sc_observe.cu); this module computes the same
quantities with numpy from exported AoS state, with the same operation order
per item and per pair, so per-pair quantities (histogram bins) match exactly
and sums match to double-precision rounding.
"""
import numpy as np


def _min_image(d, box, periodic):
    return d - box * np.rint(d / box) if periodic else d


def mark(records):
    """MSD origins: {id: float32 position} of the active items."""
    act = (records["flags"] & 1) != 0
    return {int(i): p.copy() for i, p in zip(records["id"][act], records["pos"][act])}


def observe(records, origins, box, periodic, species=0, bonds=False):
    """(msd, msd_items, mean_v2, active, bond_slots, metabolite totals) of one item set."""
    act = (records["flags"] & 1) != 0
    r = records[act]
    v = r["velocity"].astype(np.float64)
    v2 = ((v[:, 0] * v[:, 0] + v[:, 1] * v[:, 1]) + v[:, 2] * v[:, 2]).sum()
    msd_sum, msd_n = 0.0, 0
    if origins:
        ids = r["id"]
        has = np.array([int(i) in origins for i in ids], bool)
        if has.any():
            o = np.stack([origins[int(i)] for i in ids[has]]).astype(np.float64)
            p = r["pos"][has].astype(np.float64)
            d = _min_image(p - o, np.float64(box), periodic)
            msd_sum = ((d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1]) + d[:, 2] * d[:, 2]).sum()
            msd_n = int(has.sum())
    n = len(r)
    out = {"msd": msd_sum / msd_n if msd_n else 0.0, "msd_items": msd_n, "mean_v2": v2 / n if n else 0.0,
           "active": n}
    if bonds:
        out["bond_slots"] = int(np.clip(r["n_active_interactions"], 0, 8).sum())
    if species:
        out["metabolites"] = r["metabolites"][:, :species].astype(np.float64).sum(axis=0)
    return out


def pair_histogram(records, type_a, type_b, r_max, n_bins, box, periodic):
    """Distances of ordered active pairs (i, j), i != j, binned as sc_pair_histogram bins them."""
    act = (records["flags"] & 1) != 0
    r = records[act]
    a = r if type_a < 0 else r[r["type"] == type_a]
    b = r if type_b < 0 else r[r["type"] == type_b]
    counts = np.zeros(n_bins, np.uint64)
    if len(a) == 0 or len(b) == 0:
        return counts
    pa = a["pos"].astype(np.float64)
    pb = b["pos"].astype(np.float64)
    rmax = np.float64(np.float32(r_max))
    for k in range(len(a)):
        d = _min_image(pb - pa[k], np.float64(box), periodic)
        r2 = (d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1]) + d[:, 2] * d[:, 2]
        same = b["id"] == a["id"][k]
        sel = (r2 < rmax * rmax) & ~same
        bins = (np.sqrt(r2[sel]) * np.float64(n_bins) / rmax).astype(np.int64)
        bins = bins[bins < n_bins]
        counts += np.bincount(bins, minlength=n_bins).astype(np.uint64)
    return counts
