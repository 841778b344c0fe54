"""Parity checks of GPU hits against the oracle -- TEST INFRASTRUCTURE.

The bar: hit/miss, meshIndex and triangleIndex agree on >= 99.99 % of rays;
every disagreement is a tie with |dt| <= 1e-6 * t; t, b1, b2 agree within
1e-5 relative where the triangle agrees.  Any-hit results: hit/miss equals
the closest hit's, and every reported hit is a real hit of that triangle at
that t.  Used by tests/ and by bench.py's CPU leg, which checks the timed
step's hits with it."""
import numpy as np

from luxcore_gb300.workloads import NULL_INDEX

AGREE_MIN = 0.9999
TIE_REL = 1e-6
VAL_REL = 1e-5


def _rel_ok(a, b, rel):
    a = a.astype(np.float64)
    b = b.astype(np.float64)
    both_nan = np.isnan(a) & np.isnan(b)
    with np.errstate(invalid="ignore"):  # inf - inf (misses of rays with maxt = inf) compares by equality
        return both_nan | (np.abs(a - b) <= rel * np.maximum(np.abs(b), 1e-30)) | (a == b)


def compare(gpu, ref, oracle=None, rays=None):
    """Returns a dict of statistics; `ok` is the spec verdict.
    With an oracle scene and the rays, each tie is also re-tested: the GPU's
    triangle must be a real hit at the GPU's t."""
    hg = gpu["meshIndex"] != NULL_INDEX
    hr = ref["meshIndex"] != NULL_INDEX
    same = (gpu["meshIndex"] == ref["meshIndex"]) & (gpu["triangleIndex"] == ref["triangleIndex"])
    dis = ~same
    tg = gpu["t"].astype(np.float64)
    tr = ref["t"].astype(np.float64)
    with np.errstate(invalid="ignore"):
        tie = hg & hr & (np.abs(tg - tr) <= TIE_REL * np.maximum(np.abs(tr), 1e-30))
    bad_dis = dis & ~tie
    hit_same = same & hg
    vals_ok = (_rel_ok(gpu["t"][same], ref["t"][same], VAL_REL).all()
               and _rel_ok(gpu["b1"][hit_same], ref["b1"][hit_same], VAL_REL).all()
               and _rel_ok(gpu["b2"][hit_same], ref["b2"][hit_same], VAL_REL).all())
    tie_checked = True
    if oracle is not None and rays is not None:
        for i in np.nonzero(dis & tie)[0][:200]:
            ok, t, b1, b2 = oracle.triangle_hit(rays[i], int(gpu["meshIndex"][i]), int(gpu["triangleIndex"][i]))
            if not ok or t != gpu["t"][i]:
                tie_checked = False
    n = max(1, gpu.shape[0])
    agree = same.sum() / n
    out = {
        "n": int(gpu.shape[0]),
        "hit_rate": float(hr.mean()) if gpu.shape[0] else 0.0,
        "agree": float(agree),
        "ties": int((dis & tie).sum()),
        "bad_disagreements": int(bad_dis.sum()),
        "values_ok": bool(vals_ok),
        "ties_valid": bool(tie_checked),
        "bitexact_t": float((gpu["t"][hit_same] == ref["t"][hit_same]).mean()) if hit_same.any() else 1.0,
    }
    out["ok"] = bool(agree >= AGREE_MIN and out["bad_disagreements"] == 0 and vals_ok and tie_checked)
    return out


def check_anyhit(anyh, closest, oracle=None, rays=None):
    """Any-hit: hit/miss equals closest-hit hit/miss; a reported hit is a real
    hit of that triangle at that t."""
    ha = anyh["meshIndex"] != NULL_INDEX
    hc = closest["meshIndex"] != NULL_INDEX
    out = {"n": int(anyh.shape[0]), "hitmiss_agree": float((ha == hc).mean()) if anyh.shape[0] else 1.0,
           "valid": True}
    if oracle is not None and rays is not None:
        idx = np.nonzero(ha)[0]
        for i in idx[:: max(1, idx.size // 300)] if idx.size else []:
            ok, t, b1, b2 = oracle.triangle_hit(rays[i], int(anyh["meshIndex"][i]), int(anyh["triangleIndex"][i]))
            if not ok or t != anyh["t"][i] or b1 != anyh["b1"][i] or b2 != anyh["b2"][i]:
                out["valid"] = False
                break
    out["ok"] = bool(out["hitmiss_agree"] == 1.0 and out["valid"])
    return out
