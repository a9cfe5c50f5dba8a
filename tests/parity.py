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


# ---- images and light transport: disagreements classified by perturbation runs ----
#
# The CUDA kernels and the oracle draw the same sample streams (bit for bit,
# tests/test_rng.py) and run the same f32 arithmetic, but the compilers
# round differently (fused multiply-adds, the math library's last bits).
# A result can then differ only where it hangs on a decision within
# rounding of its threshold (a silhouette, a pixel boundary, a lobe or
# roulette choice) or where the path amplifies rounding continuously (a
# chain of refractions). The oracle's perturbation runs (oracle.jitter)
# nudge every traced ray by ±JITTER_SIZE relative, both ways, and show
# which results are that sensitive. A GPU result is then:
#   agree       within RTOL of the oracle's;
#   decision    the perturbation runs move the oracle's result beyond RTOL;
#   continuous  within SENSITIVITY × the largest perturbation move (the GPU's
#               rounding acting as a nudge of at most SENSITIVITY × JITTER_SIZE);
#   unexplained anything else — the tests allow none.
JITTER_SIZE = 1e-6
JITTER_RUNS = 8
RTOL = 1e-4
SENSITIVITY = 16.0


def perturbation_runs(run, runs=JITTER_RUNS, size=JITTER_SIZE):
    """run() under each perturbation run: a list of its results."""
    out = []
    for seed in range(runs):
        with oracle.jitter(seed, size):
            out.append(run())
    return out


def pixel_rel(a, b, floor=1e-3):
    """Per pixel: the largest RGB difference relative to the oracle's value (b)."""
    a, b = np.asarray(a, np.float64)[..., :3], np.asarray(b, np.float64)[..., :3]
    return np.abs(a - b).max(axis=-1) / np.maximum(np.abs(b).max(axis=-1), floor)


def classify_pixels(gpu, ref, runs, floor=1e-3):
    """Counts and masks of the four classes for an image (h×w×4 sums)."""
    d = pixel_rel(gpu, ref, floor)
    dj = np.max([pixel_rel(r, ref, floor) for r in runs], axis=0) if runs else np.zeros_like(d)
    agree = d <= RTOL
    decision = ~agree & (dj > RTOL)
    continuous = ~agree & ~decision & (d <= SENSITIVITY * dj)
    unexplained = ~agree & ~decision & ~continuous
    return {"n": int(d.size), "agree": int(agree.sum()), "decision": int(decision.sum()),
            "continuous": int(continuous.sum()), "unexplained": int(unexplained.sum()),
            "unexplained_idx": np.argwhere(unexplained)[:10].tolist(), "max_rel": float(d.max())}


EDGE_MARGIN = 1e-5


def _film(params):
    """The camera of a uniform block, for projecting points to pixel coordinates."""
    f = np.frombuffer(bytes(params), np.float32).astype(np.float64)
    u = np.frombuffer(bytes(params), np.uint32)
    return {"pos": f[0:3], "right": f[4:7], "tan": f[7], "up": f[8:11], "fwd": f[12:15], "aspect": f[15],
            "w": int(u[40]), "h": int(u[41])}


def project(film, p):
    """splat()'s film coordinates of point p (src/shaders.mjs:1452-1460), in double."""
    wo = film["pos"] - np.asarray(p, np.float64)
    wo = wo / np.linalg.norm(wo)
    cos_film = -wo @ film["fwd"]
    x = -(wo @ film["right"]) / (cos_film * film["tan"] * film["aspect"])
    y = -(wo @ film["up"]) / (cos_film * film["tan"])
    return (x + 1.0) * 0.5 * film["w"], (1.0 - y) * 0.5 * film["h"]


def classify_light_paths(gpu_photons, gpu_splats, ref, runs, params):
    """One frame's light tracing, path by path. gpu_photons: n×11 from
    raymond_light_trace (position, power, direction, then the light path's id
    and its splat's pixel as u32 bits); gpu_splats: the h×w×4 u32 sums; ref
    and runs: oracle.light_trace results (the oracle's, and under its
    perturbation runs), params the frame's uniform block. Every light path
    deposits at most one photon and makes at most one splat, at the same
    surface point.

    Photons, matched by path (a missing one counts as a difference of 1):
    agree, decision, continuous as in classify_pixels, or edge — the
    oracle's path hit a triangle or quad within EDGE_MARGIN (barycentric) of
    its edge, where rays slip between neighbours or through the seam
    depending on rounding. Splats, matched by path: the same pixel; or a
    different pixel explained by the photon's class, by a perturbation run
    moving the oracle's splat, or by the GPU photon's own position (which
    projects into the GPU's pixel, or within 1e-3 pixel of its boundary).
    Pixel sums: the GPU's sums must equal the oracle's amounts for the
    paths the GPU splatted there, within 16 units + RTOL, plus the amounts
    of paths whose difference is explained (a GPU-only splat leaves its
    pixel unbounded)."""
    NONE = 0xFFFFFFFF

    def ids_of(a):
        return np.ascontiguousarray(a).view(np.uint32).reshape(-1)

    g_ph = {int(i): gpu_photons[k, :9].astype(np.float64) for k, i in enumerate(ids_of(gpu_photons[:, 9].copy()))}
    g_px = {int(i): int(px) for i, px in zip(ids_of(gpu_photons[:, 9].copy()), ids_of(gpu_photons[:, 10].copy()))}
    o_ph = {int(i): ref["photons"][k].astype(np.float64) for k, i in enumerate(ref["photon_ids"])}
    o_sp = {int(i): ref["photon_splats"][k] for k, i in enumerate(ref["photon_ids"])}
    path_margins, first = ref["path_margins"], ref["first_id"]

    def margin(i):
        k = i - first
        return float(path_margins[k]) if 0 <= k < len(path_margins) else 1.0
    j_ph = [{int(i): r["photons"][k].astype(np.float64) for k, i in enumerate(r["photon_ids"])} for r in runs]
    j_px = [{int(i): int(r["photon_splats"][k][0]) for k, i in enumerate(r["photon_ids"])} for r in runs]

    def rel(a, b):
        if a is None or b is None:
            return 0.0 if a is None and b is None else 1.0
        return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-6))

    film = _film(params)
    out = {"paths": 0, "agree": 0, "decision": 0, "continuous": 0, "edge": 0, "unexplained": 0,
           "splat_moved": 0, "splat_unexplained": 0}
    bad, bad_splat = [], []
    cls = {}
    for i in set(g_ph) | set(o_ph):
        out["paths"] += 1
        d = rel(g_ph.get(i), o_ph.get(i))
        dj = max((rel(j.get(i), o_ph.get(i)) for j in j_ph), default=0.0)
        if d <= RTOL:
            c = "agree"
        elif dj > RTOL:
            c = "decision"
        elif d <= SENSITIVITY * dj:
            c = "continuous"
        elif margin(i) < EDGE_MARGIN:
            c = "edge"
        else:
            c = "unexplained"
            bad.append(i)
        out[c] += 1
        cls[i] = c
        pg = g_px.get(i, NONE)
        po = int(o_sp[i][0]) if i in o_sp else NONE
        if pg == po:
            continue
        out["splat_moved"] += 1
        explained = c != "agree" or any(jp.get(i, NONE) != po for jp in j_px)
        if not explained and pg != NONE and po != NONE:
            x, y = project(film, g_ph[i][:3])
            lands = int(y) * film["w"] + int(x) == pg
            near = min(x - np.floor(x), np.ceil(x) - x, y - np.floor(y), np.ceil(y) - y) < 1e-3
            explained = lands or near
        if not explained:
            out["splat_unexplained"] += 1
            bad_splat.append(i)
    # the pixel sums
    h, w = film["h"], film["w"]
    expected = np.zeros((h * w, 3), np.float64)
    budget = np.zeros(h * w, np.float64)
    for i, pg in g_px.items():
        if pg == NONE:
            continue
        if i in o_sp and int(o_sp[i][0]) != NONE:
            amount = o_sp[i][1:].astype(np.float64)
            expected[pg] += amount
            if cls[i] != "agree" or int(o_sp[i][0]) != pg:
                budget[pg] += amount.max()
        else:
            budget[pg] = np.inf
    got = np.asarray(gpu_splats, np.float64).reshape(-1, 4)[:, :3]
    dev = np.abs(got - expected).max(axis=1)
    tol = 16.0 + RTOL * expected.max(axis=1) + budget
    out["pixels_lit"] = int((got.max(axis=1) > 0).sum())
    out["pixel_unexplained"] = int((dev > tol).sum())
    out["unexplained_ids"] = sorted(bad)[:10]
    out["splat_unexplained_ids"] = sorted(bad_splat)[:10]
    out["pixel_unexplained_idx"] = np.nonzero(dev > tol)[0][:10].tolist()
    return out
