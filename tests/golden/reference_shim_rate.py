"""Single-core rate of the reference's own scan kernel body, run literally on
CPU through the test-only stand-ins of _refshim.py (one position per
simulated block), on a seeded 1 Mbp x 10-guide NGG slice at max_mismatches 4,
both strands.  Writes reference_shim_rate.json beside this file, which the
benchmark's reference arm reports as an extra CPU baseline (the reference
checkout this needs exists only in the build container).

    python tests/golden/reference_shim_rate.py --reference DIR
"""
import json
import os
import platform
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
if "--reference" in sys.argv:
    os.environ["BGO_REFERENCE_ROOT"] = sys.argv[sys.argv.index("--reference") + 1]
import _refshim  # noqa: E402

REF, F, CS, GC = _refshim.install()
from beguidedoff import encoding as E, pam as P  # noqa: E402

N_BP, N_GUIDES, K = 1_000_000, 10, 4


def main():
    rng = np.random.default_rng(31)
    seq = "".join(rng.choice(list("ACGT"), N_BP))
    packed = E.pack_2bit_to_uint32(np.array([E.NUC_TO_2BIT[c] for c in seq], dtype=np.uint8))
    comp = {"A": "T", "C": "G", "G": "C", "T": "A"}
    rc = "".join(comp[c] for c in reversed(seq))
    packed_rc = E.pack_2bit_to_uint32(np.array([E.NUC_TO_2BIT[c] for c in rc], dtype=np.uint8))
    guides = ["".join(rng.choice(list("ACGT"), 20)) for _ in range(N_GUIDES)]
    ge = np.array([E.encode_guide_64bit(np.array([E.NUC_TO_2BIT[c] for c in g], dtype=np.uint8))
                   for g in guides], dtype=np.uint64)
    pm = np.stack([P.encode_pam_mask("NGG")] * N_GUIDES).astype(np.uint8)
    pl = np.full(N_GUIDES, 3, dtype=np.uint8)
    p3 = np.ones(N_GUIDES, dtype=np.uint8)
    t0 = time.perf_counter()
    for arr, ne in ((packed, 0), (packed_rc, 3)):
        CS.search_genome_cuda(arr, N_BP, ge, pm, pl, p3, K, n_mask_packed=None, n_encoded=ne)
    dt = time.perf_counter() - t0
    comps = N_GUIDES * 2 * (N_BP - 26)
    out = {"value": comps / dt, "unit": "cmp/s", "cores": 1, "seconds": round(dt, 1),
           "sample": f"{N_BP} bp x {N_GUIDES} NGG guides, max_mismatches {K}, both strands: "
                     "beguidedoff/cuda_search.py search_chunk_kernel run literally on one CPU core "
                     "through tests/golden/_refshim.py",
           "measured_on": f"build container ({platform.machine()}), not the GPU box"}
    json.dump(out, open(os.path.join(HERE, "reference_shim_rate.json"), "w"), indent=1)
    print(json.dumps(out))


if __name__ == "__main__":
    main()
