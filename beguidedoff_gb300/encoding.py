"""2-bit DNA codec (beguidedoff/encoding.py:1-102), scalar and vectorised.

A=0 C=1 G=2 T=3; N and every other character encode as A (0).  Packed arrays
hold 16 bases per uint32, base i at bits 2*(i % 16) of word i // 16.  A guide
is a 40-bit integer with base i at bits 2*i.
"""
from typing import List

import numpy as np

NUC_TO_2BIT = {"A": 0, "C": 1, "G": 2, "T": 3, "N": 0}
BIT_TO_NUC = {0: "A", 1: "C", 2: "G", 3: "T"}
COMPLEMENT_2BIT = {0: 3, 1: 2, 2: 1, 3: 0}

# byte -> 2-bit code after upper-casing; everything but C/G/T (either case) is 0
_LUT = np.zeros(256, dtype=np.uint8)
for _c, _v in (("C", 1), ("G", 2), ("T", 3)):
    _LUT[ord(_c)] = _v
    _LUT[ord(_c.lower())] = _v
_DECODE = np.frombuffer(b"ACGT", dtype=np.uint8)


def encode_bytes(raw: bytes) -> np.ndarray:
    """Vectorised encode of an ASCII sequence (same mapping as encode_dna)."""
    return _LUT[np.frombuffer(raw, dtype=np.uint8)]


def encode_dna(seq: str) -> np.ndarray:
    return encode_bytes(seq.encode("ascii", errors="replace"))


def decode_dna(encoded: np.ndarray) -> str:
    return _DECODE[np.asarray(encoded, dtype=np.uint8) & 3].tobytes().decode()


def reverse_complement_2bit(encoded: np.ndarray) -> np.ndarray:
    return (3 - np.asarray(encoded, dtype=np.uint8)[::-1]).astype(np.uint8)


def reverse_complement_seq(seq: str) -> str:
    comp = {"A": "T", "T": "A", "G": "C", "C": "G", "N": "N"}
    return "".join(comp.get(b, b) for b in reversed(seq.upper()))


def pack_2bit_to_uint32(encoded: np.ndarray) -> np.ndarray:
    encoded = np.asarray(encoded, dtype=np.uint8)
    n_packed = (len(encoded) + 15) // 16
    padded = np.zeros(n_packed * 16, dtype=np.uint32)
    padded[: len(encoded)] = encoded
    shifts = (np.arange(16, dtype=np.uint32) * 2)[None, :]
    return np.bitwise_or.reduce(padded.reshape(n_packed, 16) << shifts, axis=1).astype(np.uint32)


def unpack_uint32_to_2bit(packed: np.ndarray, total_bp: int) -> np.ndarray:
    packed = np.asarray(packed, dtype=np.uint32)
    shifts = (np.arange(16, dtype=np.uint32) * 2)[None, :]
    return ((packed[:, None] >> shifts) & 3).astype(np.uint8).reshape(-1)[:total_bp]


def extract_window(packed: np.ndarray, start_bp: int, length: int) -> np.ndarray:
    p = np.arange(start_bp, start_bp + length, dtype=np.int64)
    return ((np.asarray(packed)[p >> 4] >> ((p & 15) * 2).astype(np.uint32)) & 3).astype(np.uint8)


def extract_windows(packed: np.ndarray, starts: np.ndarray, length: int) -> np.ndarray:
    """[n, length] 2-bit bases of windows starting at each of ``starts``."""
    p = np.asarray(starts, dtype=np.int64)[:, None] + np.arange(length, dtype=np.int64)[None, :]
    words = np.asarray(packed, dtype=np.uint32)[p >> 4]
    return ((words >> ((p & 15) * 2).astype(np.uint32)) & 3).astype(np.uint8)


def encode_guide_64bit(encoded: np.ndarray) -> int:
    val = 0
    for i, b in enumerate(np.asarray(encoded).tolist()):
        val |= int(b) << (i * 2)
    return val


def decode_guide_64bit(val: int, length: int = 20) -> np.ndarray:
    return np.array([(val >> (2 * i)) & 3 for i in range(length)], dtype=np.uint8)


def hamming_distance_2bit(val1: int, val2: int, length: int = 20) -> int:
    x = val1 ^ val2
    return ((x | (x >> 1)) & 0x5555555555).bit_count()


def mismatch_positions_2bit(val1: int, val2: int, length: int = 20) -> List[int]:
    x = val1 ^ val2
    m = (x | (x >> 1)) & 0x5555555555
    return [i + 1 for i in range(length) if (m >> (2 * i)) & 1]
