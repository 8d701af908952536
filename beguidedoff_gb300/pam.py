"""PAM encoding and validation (beguidedoff/pam.py:1-104)."""
from collections import defaultdict
from typing import Dict, List, Tuple

import numpy as np

# IUPAC code -> allowed-set nibble, bit0 = A, bit1 = C, bit2 = G, bit3 = T
IUPAC_MASK = {
    "A": 0b0001, "C": 0b0010, "G": 0b0100, "T": 0b1000,
    "R": 0b0101, "Y": 0b1010, "M": 0b0011, "K": 0b1100,
    "S": 0b0110, "W": 0b1001, "H": 0b1011, "B": 0b1110,
    "V": 0b0111, "D": 0b1101, "N": 0b1111,
}
VALID_IUPAC = set(IUPAC_MASK)
MAX_PAM_LEN = 6


def validate_pam(pam: str) -> None:
    pam = pam.upper()
    if not (1 <= len(pam) <= MAX_PAM_LEN):
        raise ValueError(f"PAM must be 1-6 characters, got {len(pam)}")
    invalid = set(pam) - VALID_IUPAC
    if invalid:
        raise ValueError(f"Invalid IUPAC codes in PAM: {invalid}")


def encode_pam_mask(pam: str) -> np.ndarray:
    pam = pam.upper()
    validate_pam(pam)
    mask = np.zeros(MAX_PAM_LEN, dtype=np.uint8)
    for i, base in enumerate(pam):
        mask[i] = IUPAC_MASK[base]
    return mask


def pam_matches_at_position(genome_2bit, position: int, pam_mask, pam_len: int) -> bool:
    for i in range(pam_len):
        gpos = position + i
        if gpos >= len(genome_2bit):
            return False
        if not ((1 << int(genome_2bit[gpos])) & int(pam_mask[i])):
            return False
    return True


def group_guides_by_pam(guides: List) -> Dict[Tuple[str, str], List]:
    groups = defaultdict(list)
    for g in guides:
        groups[(g.pam.upper(), g.pam_position.lower())].append(g)
    return dict(groups)


_EXPAND = {"A": "A", "C": "C", "G": "G", "T": "T", "R": "AG", "Y": "CT", "M": "AC", "K": "GT",
           "S": "GC", "W": "AT", "H": "ACT", "B": "CGT", "V": "ACG", "D": "AGT", "N": "ACGT"}


def all_possible_pams(pam: str) -> List[str]:
    pam = pam.upper()
    validate_pam(pam)
    out = [""]
    for c in pam:
        out = [s + b for s in out for b in _EXPAND[c]]
    return out
