"""Shared utilities against the reference's unit-test answers
(tests/test_encoding.py, test_pam.py, test_scoring.py, test_base_editing.py)."""
import numpy as np
import pytest

from beguidedoff_gb300 import encoding as E
from beguidedoff_gb300 import pam as P
from beguidedoff_gb300 import scoring as S
from beguidedoff_gb300 import base_editing as B
from beguidedoff_gb300.types import GuideInput


def test_encoding_known_answers():
    assert E.decode_dna(E.encode_dna("ACGTACGTNNACGT")) == "ACGTACGTAAACGT"
    assert E.reverse_complement_seq("ATCG") == "CGAT"
    enc = E.encode_dna("ACGT" * 10)
    assert np.array_equal(E.unpack_uint32_to_2bit(E.pack_2bit_to_uint32(enc), 40), enc)
    g = E.encode_dna("ACGTACGTACGTACGTACGT")
    assert np.array_equal(E.decode_guide_64bit(E.encode_guide_64bit(g)), g)
    va = E.encode_guide_64bit(g)
    vb = E.encode_guide_64bit(E.encode_dna("ACGTACGTACGTACGTACGA"))
    vc = E.encode_guide_64bit(E.encode_dna("TCGTACGTACGTACGTACGT"))
    assert E.hamming_distance_2bit(va, vb) == 1
    assert E.mismatch_positions_2bit(va, vb) == [20]
    assert E.mismatch_positions_2bit(va, vc) == [1]
    assert E.encode_dna("acgtRYn").tolist() == [0, 1, 2, 3, 0, 0, 0]


def test_extract_windows_matches_scalar():
    rng = np.random.default_rng(3)
    bases = rng.integers(0, 4, 1000).astype(np.uint8)
    packed = E.pack_2bit_to_uint32(bases)
    starts = rng.integers(0, 970, 50)
    w = E.extract_windows(packed, starts, 20)
    for i, s in enumerate(starts):
        assert np.array_equal(w[i], bases[s:s + 20])
        assert np.array_equal(E.extract_window(packed, int(s), 20), bases[s:s + 20])


def test_pam_known_answers():
    P.validate_pam("NGG")
    P.validate_pam("NNGRRT")
    with pytest.raises(ValueError):
        P.validate_pam("NNNNNNN")
    with pytest.raises(ValueError):
        P.validate_pam("NGX")
    m = P.encode_pam_mask("NGG")
    assert m.tolist() == [15, 4, 4, 0, 0, 0]
    pams = P.all_possible_pams("NGG")
    assert len(pams) == 4 and "AGG" in pams and "GGG" in pams
    gs = [GuideInput("g1", "A" * 20, "NGG", "3prime", 4, 8, "CBE"),
          GuideInput("g2", "A" * 20, "NNGRRT", "3prime", 4, 8, "CBE"),
          GuideInput("g3", "A" * 20, "NGG", "3prime", 4, 8, "ABE")]
    groups = P.group_guides_by_pam(gs)
    assert len(groups[("NGG", "3prime")]) == 2 and len(groups[("NNGRRT", "3prime")]) == 1


def test_pam_matches_at_position_against_allowed_sets():
    """The per-base PAM test of the reference's pam.py: every IUPAC code at
    every base, a PAM that runs past the genome's end, and NNGRRT windows."""
    codes = "ACGTRYSWKMBDHVN"
    genome = np.array([0, 1, 2, 3], dtype=np.uint8)   # A C G T
    for c in codes:
        m = P.encode_pam_mask(c)
        for pos in range(4):
            exp = "ACGT"[genome[pos]] in {"A": "A", "C": "C", "G": "G", "T": "T", "R": "AG",
                                          "Y": "CT", "S": "CG", "W": "AT", "K": "GT",
                                          "M": "AC", "B": "CGT", "D": "AGT", "H": "ACT",
                                          "V": "ACG", "N": "ACGT"}[c]
            assert P.pam_matches_at_position(genome, pos, m, 1) == exp, (c, pos)
    assert not P.pam_matches_at_position(genome, 3, P.encode_pam_mask("NN"), 2)
    g = np.array([1, 1, 2, 0, 2, 3, 0], dtype=np.uint8)   # C C G A G T A
    m = P.encode_pam_mask("NNGRRT")
    assert P.pam_matches_at_position(g, 0, m, 6)
    assert not P.pam_matches_at_position(g, 1, m, 6)


def test_cctop_known_answers():
    assert S.calculate_cctop_score([]) == 0.0
    assert abs(S.calculate_cctop_score([20]) - 1.2 ** 20) < 1e-9
    assert abs(S.calculate_cctop_score([1, 5, 10]) - (1.2 + 1.2 ** 5 + 1.2 ** 10)) < 1e-9


def test_vectorised_cctop_is_bit_exact():
    """cctop_from_masks equals Python's sum over ascending positions for
    every mask with up to 6 mismatches and a random sample of the rest."""
    from itertools import combinations

    masks = [0]
    for k in range(1, 7):
        masks += [sum(1 << (p - 1) for p in c) for c in combinations(range(1, 21), k)]
    rng = np.random.default_rng(0)
    masks += rng.integers(0, 1 << 20, 20000).tolist()
    masks = np.array(masks, dtype=np.int64)
    got = S.cctop_from_masks(masks)
    for m, v in zip(masks.tolist(), got.tolist()):
        exp = S.calculate_cctop_score([p for p in range(1, 21) if (m >> (p - 1)) & 1])
        assert v == exp


def test_base_editing_known_answers():
    seq = "ACGTACGTACGTACGTACGT"
    assert 6 in B.editable_base_in_window(seq, "CBE", 4, 8)
    pos = B.editable_base_in_window(seq, "ABE", 1, 5)
    assert 1 in pos and 5 in pos
    assert B.editable_base_in_window("G" * 20, "CBE", 1, 10) == []
    assert B.get_trinucleotide_contexts("ACGTACGT", [3]) == ["CGT"]
    assert B.has_editable_base(seq, "CBE", 4, 8)
    with pytest.raises(ValueError):
        B.editable_base_in_window(seq, "XBE", 4, 8)


def test_table_string_helpers():
    """The device-path table's window and PAM strings, mismatch-position
    strings and rounded scores equal their plain definitions."""
    from beguidedoff_gb300 import finder as F

    rng = np.random.default_rng(3)
    seq = rng.integers(0, 4, (40, 20)).astype(np.uint8)
    pam = rng.integers(0, 4, (40, 6)).astype(np.uint8)
    plen = rng.integers(1, 7, 40)
    s, p = F._decode_strings(seq, pam, plen)
    for i in range(40):
        assert s[i] == "".join("ACGT"[b] for b in seq[i])
        assert p[i] == "".join("ACGT"[b] for b in pam[i][:plen[i]])
    masks = rng.integers(0, 1 << 20, 300).astype(np.int64)
    mp = F._per_unique(masks, F._mismatch_positions, F._MM_POSITIONS)
    for m, got in zip(masks.tolist(), mp.tolist()):
        assert got == ",".join(str(i + 1) for i in range(20) if (m >> i) & 1)
    vals = S.cctop_from_masks(masks)
    r6 = F._per_unique(vals, F._round6, F._ROUND6).astype(np.float64)
    assert all(a == round(b, 6) for a, b in zip(r6.tolist(), vals.tolist()))
    assert F._decode_strings(seq[:0], pam[:0], plen[:0])[0].size == 0
