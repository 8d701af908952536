"""FASTA -> 2-bit .npz genome (beguidedoff/genome_converter.py:15-201), vectorised.

Writes the reference's format exactly: ``genome_forward`` (uint32, 16 bases
per word, LSB first, chromosomes concatenated with no separator), optional
``genome_rc`` (each chromosome reverse-complemented, same chromosome order),
``chrom_names``, ``chrom_offsets`` / ``chrom_lengths`` (int64), ``total_bp``
and optional ``n_mask`` (np.packbits big bit order over the forward strand;
only the letter N, either case, is masked; other IUPAC letters encode as A
unmasked).  The reference walks every base in Python; here each chromosome
is one table lookup.
"""
from pathlib import Path
from typing import Dict, List, Optional, Tuple

import numpy as np

from .encoding import encode_bytes, pack_2bit_to_uint32


def read_fasta(path: str) -> List[Tuple[str, bytes]]:
    """(name, sequence bytes) in file order; the name is the first word."""
    out = []
    name, chunks = None, []
    with open(path, "rb") as fh:
        for line in fh:
            line = line.rstrip(b"\r\n")
            if line.startswith(b">"):
                if name is not None:
                    out.append((name, b"".join(chunks)))
                name = line[1:].split()[0].decode() if line[1:].split() else ""
                chunks = []
            elif line:
                chunks.append(line.strip())
    if name is not None:
        out.append((name, b"".join(chunks)))
    return out


def encode_chromosomes(chroms: List[Tuple[str, bytes]], include_rc=True, include_n_mask=True,
                       device: Optional[int] = None):
    """The .npz arrays of (name, sequence) pairs; on the GPU (bgo_encode_genome)
    when ``device`` is a CUDA device index, else vectorised NumPy.  Both give
    the same bytes."""
    if device is not None and chroms and sum(len(seq) for _, seq in chroms):
        return _encode_on_device(chroms, include_rc, include_n_mask, device)
    names, offsets, lengths = [], [], []
    fwd, rc, nmask = [], [], []
    off = 0
    for name, seq in chroms:
        names.append(name)
        offsets.append(off)
        lengths.append(len(seq))
        off += len(seq)
        enc = encode_bytes(seq)
        fwd.append(enc)
        if include_n_mask:
            raw = np.frombuffer(seq, dtype=np.uint8)
            nmask.append((raw == ord("N")) | (raw == ord("n")))
        if include_rc:
            rc.append((3 - enc[::-1]).astype(np.uint8))
    full = np.concatenate(fwd) if fwd else np.zeros(0, dtype=np.uint8)
    out: Dict[str, np.ndarray] = {
        "genome_forward": pack_2bit_to_uint32(full),
        "chrom_names": np.array(names),
        "chrom_offsets": np.array(offsets, dtype=np.int64),
        "chrom_lengths": np.array(lengths, dtype=np.int64),
        "total_bp": np.int64(off),
    }
    if include_rc:
        out["genome_rc"] = pack_2bit_to_uint32(np.concatenate(rc) if rc else full)
    if include_n_mask:
        out["n_mask"] = np.packbits(np.concatenate(nmask).astype(np.uint8) if nmask
                                    else np.zeros(0, dtype=np.uint8))
    return out


def _encode_on_device(chroms, include_rc, include_n_mask, device):
    from . import _native

    lengths = np.array([len(seq) for _, seq in chroms], dtype=np.int64)
    fwd, rc, nm = _native.encode_genome(b"".join(seq for _, seq in chroms), lengths,
                                        include_rc, include_n_mask, device)
    out: Dict[str, np.ndarray] = {
        "genome_forward": fwd,
        "chrom_names": np.array([name for name, _ in chroms]),
        "chrom_offsets": np.concatenate([[0], np.cumsum(lengths)[:-1]]).astype(np.int64)
        if lengths.size else np.zeros(0, dtype=np.int64),
        "chrom_lengths": lengths,
        "total_bp": np.int64(lengths.sum()),
    }
    if include_rc:
        out["genome_rc"] = rc
    if include_n_mask:
        out["n_mask"] = nm
    return out


def convert(fasta_path: str, output_path: str, include_rc: bool = True,
            include_n_mask: bool = True, chunk_size: int = 100_000_000,
            verbose: bool = True, device: Optional[int] = None) -> None:
    chroms = read_fasta(fasta_path)
    data = encode_chromosomes(chroms, include_rc, include_n_mask, device)
    if verbose:
        print(f"  Total genome: {int(data['total_bp']):,} bp")
    np.savez_compressed(output_path, **data)
    if verbose:
        mb = Path(output_path).stat().st_size / (1024 * 1024)
        print(f"  Saved to {output_path} ({mb:.1f} MB)")


def load_genome(encoded_path: str) -> dict:
    data = np.load(encoded_path, allow_pickle=True)
    out = {
        "genome_forward": data["genome_forward"],
        "chrom_names": data["chrom_names"],
        "chrom_offsets": data["chrom_offsets"],
        "chrom_lengths": data["chrom_lengths"],
        "total_bp": int(data["total_bp"]),
    }
    if "genome_rc" in data:
        out["genome_rc"] = data["genome_rc"]
    if "n_mask" in data:
        out["n_mask"] = data["n_mask"]
    return out


def verify(encoded_path: str, fasta_path: str, sample_n: int = 10000, verbose: bool = True) -> bool:
    """Random 20-nt windows decoded from the .npz against the FASTA (N read as A)."""
    data = np.load(encoded_path, allow_pickle=True)
    seqs = dict(read_fasta(fasta_path))
    total_bp = int(data["total_bp"])
    if total_bp <= 20:
        return True
    rng = np.random.default_rng(42)
    pos = rng.integers(0, total_bp - 20, size=min(sample_n, total_bp - 20))
    offs, lens, names = data["chrom_offsets"], data["chrom_lengths"], data["chrom_names"]
    packed = data["genome_forward"]
    errors = 0
    for p in pos.tolist():
        ci = int(np.searchsorted(offs, p, side="right") - 1)
        local = p - int(offs[ci])
        if local + 20 > int(lens[ci]):
            continue
        ref = seqs[str(names[ci])][local:local + 20].decode().upper()
        got = "".join("ACGT"[(int(packed[(p + i) // 16]) >> (((p + i) % 16) * 2)) & 3]
                      for i in range(20))
        if got != ref.replace("N", "A"):
            errors += 1
    if verbose:
        print(f"  Verified {sample_n} positions: {errors} errors")
    return errors == 0
