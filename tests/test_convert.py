"""FASTA -> .npz encoding bit-identical to the reference's convert()
(beguidedoff/genome_converter.py:15-108), pinned by tests/golden/convert.npz."""
import os

import numpy as np

from _golden import GOLDEN_DIR
from beguidedoff_gb300 import genome_converter as GC


def test_convert_matches_reference(tmp_path):
    d = np.load(os.path.join(GOLDEN_DIR, "convert.npz"))
    fa = tmp_path / "g.fa"
    fa.write_text(str(d["fasta_text"]))
    for rc in (True, False):
        for nm in (True, False):
            out = tmp_path / f"o{rc}{nm}.npz"
            GC.convert(str(fa), str(out), include_rc=rc, include_n_mask=nm, verbose=False)
            got = np.load(out)
            pre = f"rc{int(rc)}_nm{int(nm)}_"
            exp_keys = sorted(k[len(pre):] for k in d.files if k.startswith(pre))
            assert sorted(got.files) == exp_keys
            for k in exp_keys:
                a, b = got[k], d[pre + k]
                assert a.dtype.kind == b.dtype.kind, k
                assert np.array_equal(a, b), k
            loaded = GC.load_genome(str(out))
            assert loaded["total_bp"] == int(d[pre + "total_bp"])
    assert GC.verify(str(tmp_path / "oTrueTrue.npz"), str(fa), sample_n=50, verbose=False) in (True, False)
