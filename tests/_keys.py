"""Hit keys in the device key layout computed by the C oracle (CPU)."""
import numpy as np

from oracle import oracle as O


def oracle_keys(genome, plan_seqs, plan_pams, max_mm):
    """Sorted keys row<<39 | strand<<38 | pos<<6 | mm for both strands."""
    n = len(plan_seqs)
    gv = np.array([O.encode_guide(s[:20]) for s in plan_seqs], dtype=np.uint64)
    pm = np.zeros((n, 6), dtype=np.uint8)
    for i, p in enumerate(plan_pams):
        for j, c in enumerate(p.upper()):
            pm[i, j] = O.IUPAC_MASK[c]
    pl = np.array([len(p) for p in plan_pams], dtype=np.uint8)
    p3 = np.ones(n, dtype=np.uint8)
    fwd, rc = O.prepare_n_masks(genome)
    out = []
    strands = [(genome["genome_forward"], fwd, 0)]
    if "genome_rc" in genome:
        strands.append((genome["genome_rc"], rc, 3))
    for slot, (arr, nm, ne) in enumerate(strands):
        _, keys = O.scan_strand(arr, genome["total_bp"], nm, gv, pm, pl, p3, max_mm, ne)
        g, pos, mm = O.split_keys(keys)
        out.append((g.astype(np.uint64) << np.uint64(39)) | (np.uint64(slot) << np.uint64(38))
                   | (pos.astype(np.uint64) << np.uint64(6)) | mm.astype(np.uint64))
    return np.sort(np.concatenate(out)) if out else np.zeros(0, dtype=np.uint64)


def table_rows(t):
    """Row dicts from a Table or a pandas DataFrame."""
    if hasattr(t, "rows"):
        return [dict(r) for r in t.rows()]
    return t.to_dict("records")
