"""Per-ray hit parity between the CUDA path and the oracle's Scene.raycast.

A ray passes when both report the same leaf-order primitive. Otherwise:
* tie: both primitives are hit in double and their distances agree to
  |Δt|/t ≤ 1e-5 (the reference's grazing-tie allowance);
* silhouette: one of the two primitives is crossed within f32 rounding of
  its edge (a sphere's discriminant within f32 cancellation error of zero, a
  triangle's or quad's crossing within 1e-4 of an edge in barycentric
  terms, a box's entry and exit within 1e-4 relative), so f32 and double
  legitimately disagree on hit-or-miss; the reference tolerates 0.5% of
  pixels disagreeing at silhouettes (tests/browser/app.test.mjs:154-155);
* wrong: anything else — never allowed.
"""

import numpy as np

import oracle

NONE = 0xFFFFFFFF
TIE_RTOL = 1e-5
EDGE_TOL = 1e-4
EPS32 = 2.0 ** -23


def grazing(packed, p, o, d) -> bool:
    """Whether the ray crosses primitive p within f32 rounding of its edge."""
    rec = packed.primitives.reshape(-1, 16)[p]
    f = rec.view(np.float32).astype(np.float64)
    kind = int(rec[0])
    if kind == 0:  # sphere: discriminant near zero relative to its terms
        oc = o - f[4:7]
        a, hb, c = d @ d, oc @ d, oc @ oc - f[7] * f[7]
        disc = hb * hb - a * c
        return abs(disc) <= 64 * EPS32 * (hb * hb + abs(a * c))
    if kind == 1:  # quad: edge coordinates near 0 or 1
        q, qu, qv = f[4:7], f[8:11], f[12:15]
        n = np.cross(qu, qv)
        denom = n @ d
        if abs(denom) < 1e-12:
            return True
        t = n @ (q - o) / denom
        h = o + d * t - q
        nn = n @ n
        alpha, beta = n @ np.cross(h, qv) / nn, n @ np.cross(qu, h) / nn
        return min(abs(alpha), abs(alpha - 1), abs(beta), abs(beta - 1)) < EDGE_TOL
    if kind == 2:  # box: entry and exit nearly equal (crossing an edge or corner)
        rows = f[4:16].reshape(3, 4)
        lo = rows[:, :3] @ o + rows[:, 3]
        ld = rows[:, :3] @ d
        with np.errstate(divide="ignore", invalid="ignore"):
            t0, t1 = (-1 - lo) / ld, (1 - lo) / ld
        ok = ~np.isnan(t0) & ~np.isnan(t1)
        tn, tf = np.max(np.minimum(t0, t1)[ok]), np.min(np.maximum(t0, t1)[ok])
        return abs(tf - tn) <= EDGE_TOL * max(abs(tn), abs(tf), 1e-12)
    if kind == 3:  # triangle: barycentrics near an edge
        v0, v1, v2 = f[4:7], f[8:11], f[12:15]
        e1, e2 = v1 - v0, v2 - v0
        pv = np.cross(d, e2)
        det = e1 @ pv
        if abs(det) < 1e-12:
            return True
        tv = o - v0
        bu = tv @ pv / det
        bv = d @ np.cross(tv, e1) / det
        return min(abs(bu), abs(bv), abs(1 - bu - bv), abs(bu - 1), abs(bv - 1)) < EDGE_TOL
    return False


def classify(packed, rays, gpu_prim, gpu_t, ref):
    rays = rays.reshape(-1, 6)
    same = gpu_prim == ref["prim"]
    ties, silhouettes, hit_miss, wrong = [], [], [], []
    for i in np.nonzero(~same)[0]:
        gp, rp = int(gpu_prim[i]), int(ref["prim"][i])
        o = rays[i, :3].astype(np.float64)
        d = rays[i, 3:].astype(np.float64)
        if gp != NONE and rp != NONE:
            g = oracle.intersect_double(packed, gp, o, d)
            if g is not None and abs(g[0] - ref["t"][i]) <= TIE_RTOL * ref["t"][i]:
                ties.append(i)
                continue
        if (gp != NONE and grazing(packed, gp, o, d)) or (rp != NONE and grazing(packed, rp, o, d)):
            (hit_miss if NONE in (gp, rp) else silhouettes).append(i)
        else:
            wrong.append(i)
    both_hit = (gpu_prim != NONE) & (ref["prim"] != NONE) & same
    t_rel = np.abs(gpu_t[both_hit].astype(np.float64) - ref["t"][both_hit]) / np.maximum(ref["t"][both_hit], 1e-12)
    return {
        "n": len(gpu_prim), "same": int(same.sum()), "ties": len(ties), "silhouettes": len(silhouettes),
        "hit_miss": len(hit_miss), "wrong": len(wrong), "wrong_idx": wrong[:10],
        "max_t_rel": float(t_rel.max()) if t_rel.size else 0.0,
    }
