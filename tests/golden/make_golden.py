"""Generate golden vectors by running the reference's own extensive path on CPU.

Usage (in a container that has the reference checkout; the GPU machine does not):

    python tests/golden/make_golden.py --reference DIR [--only NAME ...] [--workers N]

Each case writes ``tests/golden/<name>.npz`` holding

* the genome exactly as the reference's ``genome_converter.convert``
  (beguidedoff/genome_converter.py:15-108) wrote it from a seeded FASTA,
* the guide rows fed to ``beguidedoff.finder.beguidedoff.search``
  (beguidedoff/finder.py:474-566) and the search parameters,
* the output table rows the reference returned (one column per array),
* every raw call into ``search_genome_cuda`` (beguidedoff/cuda_search.py:384)
  with its inputs and its per-guide ``(position, mismatches)`` lists, so the
  kernel seam is pinned independently of the host post-processing.

The reference runs through the stand-ins in ``_refshim.py`` (its Numba kernel
body executes literally on CPU, one position per simulated block).  Inputs are
generated here from fixed seeds; the fixtures store the generated data itself,
so the tests never need this script or the reference.
"""
import argparse
import json
import os
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
if "--reference" in sys.argv:
    os.environ["BGO_REFERENCE_ROOT"] = sys.argv[sys.argv.index("--reference") + 1]
import _refshim  # noqa: E402

REF, F, CS, GC = _refshim.install()
from beguidedoff.types import GuideInput  # noqa: E402

_COMP = {"A": "T", "C": "G", "G": "C", "T": "A", "N": "N"}
_TABLE_COLS = [
    "guide_rna_sequence", "base_editor", "ot_rank", "ot_chromosome", "ot_position",
    "ot_strand", "ot_sequence", "ot_pam", "n_mismatches", "mismatch_positions",
    "score", "n_offtargets_below_threshold",
]
_RESOLVE = {"A": "A", "C": "C", "G": "G", "T": "T", "R": "AG", "Y": "CT", "M": "AC",
            "K": "GT", "S": "CG", "W": "AT", "H": "ACT", "B": "CGT", "V": "ACG",
            "D": "AGT", "N": "ACGT"}


def revcomp(s):
    return "".join(_COMP[c] for c in reversed(s))


def rand_seq(rng, n, p=None):
    return "".join(rng.choice(list("ACGT"), size=n, p=p))


def resolve_pam(rng, pam):
    return "".join(rng.choice(list(_RESOLVE[c])) for c in pam)


def mutate(rng, seq, n_sub, positions=None):
    s = list(seq)
    pos = positions if positions is not None else rng.choice(len(s), size=n_sub, replace=False)
    for p in pos:
        s[p] = rng.choice([b for b in "ACGT" if b != s[p]])
    return "".join(s)


def plant(rng, chrom, guide, pam, n_sub, strand, at=None):
    """Overwrite a site (guide with n_sub substitutions + concrete PAM)."""
    site = mutate(rng, guide, n_sub) + resolve_pam(rng, pam)
    if strand == "-":
        site = revcomp(site)
    if at is None:
        at = int(rng.integers(0, len(chrom) - len(site)))
    return chrom[:at] + site + chrom[at + len(site):]


def add_n_runs(rng, chrom, frac, lo, hi):
    s = list(chrom)
    target = int(frac * len(s))
    done = 0
    while done < target:
        run = int(rng.integers(lo, hi + 1))
        at = int(rng.integers(0, max(1, len(s) - run)))
        s[at:at + run] = ["N"] * min(run, len(s) - at)
        done += run
    return "".join(s)


def write_fasta(path, chroms):
    with open(path, "w") as fh:
        for name, seq in chroms.items():
            fh.write(f">{name}\n")
            for i in range(0, len(seq), 60):
                fh.write(seq[i:i + 60] + "\n")


class Recorder:
    """Wraps ``finder.search_genome_cuda`` to record every raw kernel call."""

    def __init__(self):
        self.calls = []
        self._orig = F.search_genome_cuda

    def __enter__(self):
        def wrapped(genome_packed, total_bp, guide_encoded, pam_masks, pam_lens,
                    pam_3prime, max_mismatches, **kw):
            out = self._orig(genome_packed, total_bp, guide_encoded, pam_masks, pam_lens,
                             pam_3prime, max_mismatches, **kw)
            res, ovf, cnt = out if kw.get("return_overflow") else (out, {}, {})
            gi, pos, mm = [], [], []
            for g, lst in res.items():
                for p, m in lst:
                    gi.append(g)
                    pos.append(p)
                    mm.append(m)
            self.calls.append(dict(
                n_encoded=int(kw.get("n_encoded", 0)),
                results_per_guide=int(kw.get("results_per_guide", 10240)),
                max_mismatches=int(max_mismatches),
                guide_encoded=np.asarray(guide_encoded, dtype=np.uint64),
                pam_masks=np.asarray(pam_masks, dtype=np.uint8),
                pam_lens=np.asarray(pam_lens, dtype=np.uint8),
                pam_3prime=np.asarray(pam_3prime, dtype=np.uint8),
                hit_guide=np.asarray(gi, dtype=np.int32),
                hit_pos=np.asarray(pos, dtype=np.int64),
                hit_mm=np.asarray(mm, dtype=np.int8),
                counts=np.asarray([cnt.get(g, 0) for g in range(len(guide_encoded))],
                                  dtype=np.int64),
            ))
            return out

        F.search_genome_cuda = wrapped
        return self

    def __exit__(self, *a):
        F.search_genome_cuda = self._orig


def guide_arrays(guides):
    def col(name, fill):
        return [fill if getattr(g, name) is None else getattr(g, name) for g in guides]
    return {
        "g_id": np.array([g.guide_id for g in guides]),
        "g_seq": np.array([g.guide_seq for g in guides]),
        "g_pam": np.array([g.pam for g in guides]),
        "g_ws": np.array([g.edit_window_start for g in guides], dtype=np.int64),
        "g_we": np.array([g.edit_window_end for g in guides], dtype=np.int64),
        "g_editor": np.array([g.editor_type for g in guides]),
        "g_ot_chrom": np.array(col("on_target_chrom", "")),
        "g_ot_pos": np.array(col("on_target_pos", -1), dtype=np.int64),
        "g_ot_strand": np.array(col("on_target_strand", "")),
        "g_base_editor": np.array(col("base_editor", "")),
    }


def table_arrays(df, prefix):
    rows = df.rows
    out = {}
    for c in _TABLE_COLS:
        vals = [r[c] for r in rows]
        if c in ("ot_rank", "ot_position", "n_mismatches", "n_offtargets_below_threshold"):
            out[prefix + c] = np.array(vals, dtype=np.int64)
        elif c == "score":
            out[prefix + c] = np.array(vals, dtype=np.float64)
        else:
            out[prefix + c] = np.array(vals, dtype=str)
    return out


def run_case(name, chroms, guides, runs, *, include_n_mask=True, max_mm=4, n_top=3,
             results_per_guide=10240, max_results_per_guide=None):
    """Convert, search once per entry of ``runs`` and save one fixture."""
    t0 = time.time()
    with tempfile.TemporaryDirectory() as td:
        fa = os.path.join(td, "genome.fa")
        npz = os.path.join(td, "genome.npz")
        write_fasta(fa, chroms)
        GC.convert(fa, npz, include_n_mask=include_n_mask, verbose=False)
        gd = GC.load_genome(npz)
        finder = REF.beguidedoff(genome_path=npz, max_mismatches=max_mm, n_top_offtargets=n_top,
                                 results_per_guide=results_per_guide,
                                 max_results_per_guide=max_results_per_guide, device="cuda:0")
        fixture = {
            "genome_forward": gd["genome_forward"],
            "genome_rc": gd["genome_rc"],
            "chrom_names": np.array([str(c) for c in gd["chrom_names"]]),
            "chrom_offsets": gd["chrom_offsets"],
            "chrom_lengths": gd["chrom_lengths"],
            "total_bp": np.int64(gd["total_bp"]),
        }
        if "n_mask" in gd:
            fixture["n_mask"] = gd["n_mask"]
        fixture.update(guide_arrays(guides))
        meta = {"name": name, "max_mismatches": max_mm, "n_top_offtargets": n_top,
                "results_per_guide": results_per_guide,
                "max_results_per_guide": max_results_per_guide, "runs": [], "raw_calls": 0}
        raw_index = 0
        for ri, run in enumerate(runs):
            with Recorder() as rec:
                with _refshim_capture_warnings() as warns:
                    df = finder.search(guides=guides, verbose=False, **run["kwargs"])
            fixture.update(table_arrays(df, f"r{ri}_"))
            run_meta = {"kwargs": run["kwargs"], "n_rows": len(df), "warnings": warns.messages,
                        "raw_calls": list(range(raw_index, raw_index + len(rec.calls)))}
            for c in rec.calls:
                for k, v in c.items():
                    fixture[f"raw{raw_index}_{k}"] = np.asarray(v)
                raw_index += 1
            meta["runs"].append(run_meta)
        meta["raw_calls"] = raw_index
        fixture["meta_json"] = np.array(json.dumps(meta))
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **fixture)
    print(f"{name}: {[r['n_rows'] for r in meta['runs']]} rows, {raw_index} raw calls, "
          f"{time.time() - t0:.1f}s")


class _refshim_capture_warnings:
    def __enter__(self):
        import logging

        self.messages = []
        outer = self

        class H(logging.Handler):
            def emit(self, record):
                outer.messages.append(record.getMessage())

        self.h = H(level=logging.WARNING)
        self.logger = logging.getLogger("beguidedoff")
        self.logger.addHandler(self.h)
        self.old_level = self.logger.level
        self.logger.setLevel(logging.WARNING)
        return self

    def __exit__(self, *a):
        self.logger.removeHandler(self.h)
        self.logger.setLevel(self.old_level)


# ----------------------------------------------------------------------------
# cases
# ----------------------------------------------------------------------------
def case_planted_ngg():
    """Small stand-in for the 10 Mbp plain configuration: 2 chromosomes, 1% N
    runs, 10 NGG guides x 20 planted sites with 0-4 substitutions, both strands."""
    rng = np.random.default_rng(101)
    lens = (26_000, 14_000)
    chroms = {f"chr{i + 1}": rand_seq(rng, n) for i, n in enumerate(lens)}
    chroms = {k: add_n_runs(rng, v, 0.01, 100, 400) for k, v in chroms.items()}
    guides_seq = [rand_seq(rng, 20) for _ in range(10)]
    names = list(chroms)
    for g in guides_seq:
        for _ in range(20):
            c = names[int(rng.integers(0, 2))]
            chroms[c] = plant(rng, chroms[c], g, "NGG", int(rng.integers(0, 5)),
                              "+" if rng.random() < 0.5 else "-")
    guides = []
    for i, g in enumerate(guides_seq):
        et = "ABE" if i % 2 == 0 else "CBE"
        guides.append(GuideInput(f"row_{i}", g, "NGG", "3prime", 4, 8, et,
                                 base_editor="ABE8e" if et == "ABE" else "TadCBEd"))
    # one exact on-target on each strand, excluded by coordinates
    c1 = chroms["chr1"]
    ot_plus = guides_seq[1] + "TGG"
    chroms["chr1"] = c1[:5000] + ot_plus + c1[5000 + 23:]
    ot_minus = revcomp(guides_seq[2] + "AGG")
    c1 = chroms["chr1"]
    chroms["chr1"] = c1[:9000] + ot_minus + c1[9000 + 23:]
    guides[1] = GuideInput("row_1", guides_seq[1], "NGG", "3prime", 4, 8, "CBE",
                           on_target_chrom="chr1", on_target_pos=5001, on_target_strand="+",
                           base_editor="TadCBEd")
    guides[2] = GuideInput("row_2", guides_seq[2], "NGG", "3prime", 2, 13, "ABE",
                           on_target_chrom="chr1", on_target_pos=9023, on_target_strand="-",
                           base_editor="ABE8e")
    # duplicate scan key with a different editor (dedup maps both rows)
    guides.append(GuideInput("row_10", guides_seq[0], "NGG", "3prime", 5, 8, "CBE"))
    runs = [
        {"kwargs": {"return_all": True}},
        {"kwargs": {"return_all": False, "count_score_threshold": 5.0}},
        {"kwargs": {"return_all": False, "count_score_threshold": 40.0}},
    ]
    run_case("planted_ngg", chroms, guides, runs, max_mm=4, n_top=3)


def case_mixed_pam():
    """PAM families NGG/NG/NNGRRT/NNNRRT/NRN plus exotic and edge PAMs, three
    chromosomes (one shorter than a site) and sites straddling junctions."""
    rng = np.random.default_rng(202)
    chroms = {"chrA": rand_seq(rng, 9_000), "chrB": rand_seq(rng, 24), "chrC": rand_seq(rng, 7_000)}
    pams = ["NGG", "NG", "NNGRRT", "NNNRRT", "NRN", "TTTV", "SGG", "WGG", "G", "NNNNNN",
            "NAG", "KYM", "BDH"]
    guides_seq = [rand_seq(rng, 20) for _ in pams]
    for g, pam in zip(guides_seq, pams):
        for _ in range(6):
            c = "chrA" if rng.random() < 0.6 else "chrC"
            chroms[c] = plant(rng, chroms[c], g, pam, int(rng.integers(0, 6)),
                              "+" if rng.random() < 0.5 else "-")
    # junction straddlers: a forward site across chrA|chrB|chrC and a reverse one
    g0 = guides_seq[0]
    site = g0 + "AGG"
    chroms["chrA"] = chroms["chrA"][:-10] + site[:10]
    chroms["chrB"] = site[10:] + chroms["chrB"][13:16] + chroms["chrB"][16:]
    g1 = guides_seq[1]
    rsite = revcomp(mutate(rng, g1, 1) + "TG")
    chroms["chrC"] = rsite[8:] + chroms["chrC"][len(rsite) - 8:]
    chroms["chrB"] = chroms["chrB"][:-8] + rsite[:8]
    guides = [GuideInput(f"row_{i}", g, pam, "3prime", 3, 9, "CBE" if i % 3 else "ABE")
              for i, (g, pam) in enumerate(zip(guides_seq, pams))]
    # same scan key as row_2 (dedup) with a different editor and window
    guides.append(GuideInput("row_x", guides_seq[2], "NNGRRT", "3prime", 1, 20, "CGE"))
    runs = [{"kwargs": {"return_all": True}},
            {"kwargs": {"return_all": False, "count_score_threshold": 10.0}}]
    run_case("mixed_pam", chroms, guides, runs, max_mm=5, n_top=5)


def case_n_gate():
    """The reference's N-gate genomes (tests/test_extensive_gpu.py:116-204)
    concatenated as chromosomes, plus a random genome with many short N runs."""
    rng = np.random.default_rng(303)
    chroms = {
        "blk": ("G" * 40 + "T" * 20 + "TTT" + "G" * 40 + "N" * 500 + "G" * 40 + "A" * 20
                + "AAA" + "G" * 40),
        "adj": "G" * 30 + "N" * 10 + "CCC" + "T" * 20 + "G" * 30,
        "rnd": add_n_runs(rng, rand_seq(rng, 6_000), 0.08, 1, 30),
    }
    polya = "A" * 20
    for _ in range(10):
        chroms["rnd"] = plant(rng, chroms["rnd"], "AAAATAAAAAAATAAAAAAA", "NGG",
                              int(rng.integers(0, 3)), "+" if rng.random() < 0.5 else "-")
    guides = [
        GuideInput("polyA", polya, "AAA", "3prime", 4, 8, "CBE"),
        GuideInput("polyT", "T" * 20, "TTT", "3prime", 4, 8, "CBE"),
        GuideInput("polyA_ngg", polya, "NGG", "3prime", 4, 8, "CBE"),
        GuideInput("at_rich", "AAAATAAAAAAATAAAAAAA", "NGG", "3prime", 1, 20, "ABE"),
        GuideInput("polyA_nnn", polya, "NNN", "3prime", 1, 20, "ABE"),
    ]
    runs = [{"kwargs": {"return_all": True}}]
    run_case("n_gate", chroms, guides, runs, max_mm=4, n_top=3)
    run_case("n_gate_nomask", chroms, guides, runs, include_n_mask=False, max_mm=4, n_top=3)


def case_overflow():
    """12,000 copies of a 1-mismatch site (tests/test_extensive_gpu.py:38-107):
    the exact count, and the truncation at a 10,240-hit ceiling."""
    guide = "ACGTACGTACGTACGTACGT"
    unit = "T" + guide[1:] + "AGG"
    chroms = {"chr1": unit * 12_000 + "A" * 30}
    guides = [GuideInput("g1", guide, "NGG", "3prime", 4, 8, "CBE")]
    runs = [{"kwargs": {"return_all": False, "count_score_threshold": 5.0}}]
    run_case("overflow", chroms, guides, runs, max_mm=4, n_top=3)
    runs = [{"kwargs": {"return_all": True}}]
    run_case("overflow_capped", chroms, guides, runs, max_mm=4, n_top=3,
             max_results_per_guide=10240)


def case_repeats():
    """Repeat families at ~10% divergence, half the guides from the consensus,
    max_mismatches=6: thousands of hits, many ties in score."""
    rng = np.random.default_rng(404)
    fams = [rand_seq(rng, 300) for _ in range(3)]
    parts = []
    for _ in range(60):
        parts.append(rand_seq(rng, int(rng.integers(20, 200))))
        f = fams[int(rng.integers(0, 3))]
        copy = mutate(rng, f, 30)
        parts.append(copy if rng.random() < 0.5 else revcomp(copy))
    chroms = {"r1": "".join(parts[:60]), "r2": "".join(parts[60:])}
    guides_seq = []
    for f in fams:
        for _ in range(2):
            while True:
                at = int(rng.integers(0, 277))
                if f[at + 21:at + 23] in ("GG", "AG"):
                    break
            guides_seq.append(f[at:at + 20])
    guides_seq += [rand_seq(rng, 20) for _ in range(4)]
    guides = [GuideInput(f"row_{i}", g, "NRG", "3prime", 2, 13, ["ABE", "CBE", "CGE"][i % 3])
              for i, g in enumerate(guides_seq)]
    runs = [{"kwargs": {"return_all": True}},
            {"kwargs": {"return_all": False, "count_score_threshold": 30.0}}]
    run_case("repeats", chroms, guides, runs, max_mm=6, n_top=4)


def case_many_guides():
    """2,100 scan keys (> one launch of 2,048) on a 3 kbp genome
    (tests/test_extensive_gpu.py:207-233)."""
    from itertools import product

    rng = np.random.default_rng(7)
    genome = list(rand_seq(rng, 3_000))
    guides = [GuideInput(f"g{i}", "ACGTACGTACGTAC" + "".join(p), "NGG", "3prime", 4, 8, "CBE")
              for i, p in enumerate(product("ACGT", repeat=6))][:2_100]
    planted = guides[137]
    for pos in (500, 1_500, 2_500):
        genome[pos:pos + 20] = list(planted.guide_seq)
        genome[pos + 20:pos + 23] = list("AGG")
    chroms = {"chr1": "".join(genome)}
    runs = [{"kwargs": {"return_all": False}}]
    run_case("many_guides", chroms, guides, runs, max_mm=4, n_top=3)


def case_seam_5prime():
    """Direct calls of the kernel seam ``search_genome_cuda`` with 5' PAMs,
    exotic codes, a zero-length PAM and max_mismatches 0..3 on both strands."""
    rng = np.random.default_rng(505)
    chroms = {"c1": add_n_runs(rng, rand_seq(rng, 3_000), 0.05, 3, 40),
              "c2": rand_seq(rng, 1_500)}
    pam_list = ["TTTV", "TTN", "NGG", "V", "YG", ""]
    guides_seq = [rand_seq(rng, 20) for _ in pam_list]
    for g, pam in zip(guides_seq, pam_list):
        for _ in range(5):
            c = "c1" if rng.random() < 0.6 else "c2"
            site = resolve_pam(rng, pam) + mutate(rng, g, int(rng.integers(0, 3)))
            if rng.random() < 0.5:
                site = revcomp(site)
            at = int(rng.integers(0, len(chroms[c]) - len(site)))
            chroms[c] = chroms[c][:at] + site + chroms[c][at + len(site):]
    t0 = time.time()
    fixture = {}
    with tempfile.TemporaryDirectory() as td:
        fa = os.path.join(td, "g.fa")
        npz = os.path.join(td, "g.npz")
        write_fasta(fa, chroms)
        GC.convert(fa, npz, verbose=False)
        gd = GC.load_genome(npz)
        for k in ("genome_forward", "genome_rc", "chrom_offsets", "chrom_lengths", "n_mask"):
            fixture[k] = gd[k]
        fixture["chrom_names"] = np.array([str(c) for c in gd["chrom_names"]])
        fixture["total_bp"] = np.int64(gd["total_bp"])
        from beguidedoff.pam import encode_pam_mask
        from beguidedoff.encoding import encode_dna, encode_guide_64bit

        n = len(pam_list)
        gv = np.array([encode_guide_64bit(encode_dna(g)) for g in guides_seq], dtype=np.uint64)
        masks = np.zeros((n, 6), dtype=np.uint8)
        for i, pam in enumerate(pam_list):
            if pam:
                masks[i] = encode_pam_mask(pam)
        lens = np.array([len(p) for p in pam_list], dtype=np.uint8)
        calls = 0
        # n_mask as prepared by finder._prepare_n_masks (little bit order + 16 B pad)
        bits = np.unpackbits(gd["n_mask"], bitorder="big", count=int(gd["total_bp"]))
        nm_fwd = np.pad(np.packbits(bits, bitorder="little"), (0, 16))
        rc_bits = np.empty_like(bits)
        for off, ln in zip(gd["chrom_offsets"], gd["chrom_lengths"]):
            rc_bits[off:off + ln] = bits[off:off + ln][::-1]
        nm_rc = np.pad(np.packbits(rc_bits, bitorder="little"), (0, 16))
        for three in (0, 1):
            for strand, arr, nm, ne in (("+", gd["genome_forward"], nm_fwd, 0),
                                        ("-", gd["genome_rc"], nm_rc, 3)):
                for max_mm in (0, 3):
                    p3 = np.full(n, three, dtype=np.uint8)
                    res, ovf, cnt = CS.search_genome_cuda(
                        arr, int(gd["total_bp"]), gv, masks, lens, p3, max_mm,
                        return_overflow=True, results_per_guide=7, n_mask_packed=nm,
                        n_encoded=ne)
                    gi, pos, mm = [], [], []
                    for g, lst in res.items():
                        for p, m in lst:
                            gi.append(g)
                            pos.append(p)
                            mm.append(m)
                    pre = f"raw{calls}_"
                    fixture[pre + "strand"] = np.array(strand)
                    fixture[pre + "n_encoded"] = np.int64(ne)
                    fixture[pre + "pam_3prime"] = p3
                    fixture[pre + "max_mismatches"] = np.int64(max_mm)
                    fixture[pre + "results_per_guide"] = np.int64(7)
                    fixture[pre + "hit_guide"] = np.array(gi, dtype=np.int32)
                    fixture[pre + "hit_pos"] = np.array(pos, dtype=np.int64)
                    fixture[pre + "hit_mm"] = np.array(mm, dtype=np.int8)
                    fixture[pre + "counts"] = np.array([cnt[g] for g in range(n)], dtype=np.int64)
                    fixture[pre + "overflow"] = np.array([ovf[g] for g in range(n)], dtype=bool)
                    calls += 1
        fixture["guide_encoded"] = gv
        fixture["pam_masks"] = masks
        fixture["pam_lens"] = lens
        fixture["meta_json"] = np.array(json.dumps({"name": "seam_5prime", "raw_calls": calls}))
    np.savez_compressed(os.path.join(HERE, "seam_5prime.npz"), **fixture)
    print(f"seam_5prime: {calls} raw calls, {time.time() - t0:.1f}s")


def case_convert():
    """FASTA -> .npz encoding with lower case, N, other IUPAC letters and
    several chromosomes (beguidedoff/genome_converter.py:15-108)."""
    rng = np.random.default_rng(606)
    chroms = {}
    for i, n in enumerate((37, 1, 100, 16, 250)):
        s = list(rand_seq(rng, n))
        for j in range(n):
            r = rng.random()
            if r < 0.1:
                s[j] = "N"
            elif r < 0.15:
                s[j] = s[j].lower()
            elif r < 0.18:
                s[j] = rng.choice(list("RYKMSWn"))
        chroms[f"s{i}"] = "".join(s)
    fixture = {}
    with tempfile.TemporaryDirectory() as td:
        fa = os.path.join(td, "g.fa")
        write_fasta(fa, chroms)
        fixture["fasta_text"] = np.array(open(fa).read())
        for rc in (True, False):
            for nm in (True, False):
                npz = os.path.join(td, f"g{rc}{nm}.npz")
                GC.convert(fa, npz, include_rc=rc, include_n_mask=nm, verbose=False)
                d = np.load(npz, allow_pickle=True)
                for k in d.files:
                    fixture[f"rc{int(rc)}_nm{int(nm)}_{k}"] = d[k]
    np.savez_compressed(os.path.join(HERE, "convert.npz"), **fixture)
    print("convert: ok")


def case_sacas9_21nt():
    """21-nt guides of the SaCas9 families (NNGRRT, NNNRRT) beside 20-nt NGG
    guides.  The reference packs a 21-nt guide into 42 bits but compares only
    its first 20 bases (40-bit mask) and tests the PAM right after them
    (beguidedoff/encoding.py:70-75, cuda_search.py:239-275); sites are planted
    both as the first 20 bases + PAM and as all 21 bases + PAM."""
    rng = np.random.default_rng(2121)
    chroms = {"chr1": rand_seq(rng, 30_000), "chr2": rand_seq(rng, 20_000)}
    chroms = {k: add_n_runs(rng, v, 0.01, 50, 300) for k, v in chroms.items()}
    specs = [(21, "NNGRRT"), (21, "NNNRRT"), (21, "NNGRRT"), (20, "NGG"), (21, "NGG")]
    guides_seq = [rand_seq(rng, n) for n, _ in specs]
    names = list(chroms)
    for g, (n, pam) in zip(guides_seq, specs):
        for k in range(8):
            c = names[int(rng.integers(0, 2))]
            core = g[:20] if k % 2 == 0 else g
            chroms[c] = plant(rng, chroms[c], core, pam, int(rng.integers(0, 4)),
                              "+" if rng.random() < 0.5 else "-")
    guides = []
    for i, (g, (n, pam)) in enumerate(zip(guides_seq, specs)):
        et = ("ABE", "CBE", "CGE")[i % 3]
        guides.append(GuideInput(f"sa_{i}", g, pam, "3prime", 3, 9, et))
    runs = [{"kwargs": {"return_all": True, "count_score_threshold": 5.0}},
            {"kwargs": {"return_all": False}}]
    run_case("sacas9_21nt", chroms, guides, runs, max_mm=4, n_top=3)


def case_config1():
    """The plain CPU-runnable configuration at its stated size (10 Mbp, 2
    chromosomes, 1% N in runs of 100-5,000 bp, 10 NGG guides x 20 planted
    sites with 0-4 substitutions, ABE window 4-8, max_mismatches 4), generated
    by config1.py.  The fixture keeps the hashes of the genome arrays the
    reference's converter wrote, not the arrays."""
    import config1 as C1

    t0 = time.time()
    chroms, guides_seq, on = C1.generate()
    guides = C1.guide_inputs(GuideInput, guides_seq, on)
    runs = [{"kwargs": {"return_all": True, "count_score_threshold": 5.0}},
            {"kwargs": {"return_all": False, "count_score_threshold": 40.0}}]
    with tempfile.TemporaryDirectory() as td:
        fa = os.path.join(td, "genome.fa")
        npz = os.path.join(td, "genome.npz")
        with open(fa, "w") as fh:
            for name, seq in chroms:
                fh.write(f">{name}\n")
                text = seq.decode()
                for i in range(0, len(text), 60):
                    fh.write(text[i:i + 60] + "\n")
        GC.convert(fa, npz, include_n_mask=True, verbose=False)
        gd = GC.load_genome(npz)
        fixture = {
            "chrom_names": np.array([str(c) for c in gd["chrom_names"]]),
            "chrom_offsets": gd["chrom_offsets"],
            "chrom_lengths": gd["chrom_lengths"],
            "total_bp": np.int64(gd["total_bp"]),
            "sha_forward": np.array(C1.digest(gd["genome_forward"])),
            "sha_rc": np.array(C1.digest(gd["genome_rc"])),
            "sha_n_mask": np.array(C1.digest(gd["n_mask"])),
        }
        fixture.update(guide_arrays(guides))
        finder = REF.beguidedoff(genome_path=npz, max_mismatches=C1.MAX_MISMATCHES,
                                 n_top_offtargets=3, device="cuda:0")
        meta = {"name": "config1", "max_mismatches": C1.MAX_MISMATCHES, "n_top_offtargets": 3,
                "results_per_guide": 10240, "max_results_per_guide": None, "runs": [],
                "raw_calls": 0}
        for ri, run in enumerate(runs):
            with _refshim_capture_warnings() as warns:
                df = finder.search(guides=guides, verbose=False, **run["kwargs"])
            fixture.update(table_arrays(df, f"r{ri}_"))
            meta["runs"].append({"kwargs": run["kwargs"], "n_rows": len(df),
                                 "warnings": warns.messages, "raw_calls": []})
        fixture["meta_json"] = np.array(json.dumps(meta))
    np.savez_compressed(os.path.join(HERE, "config1.npz"), **fixture)
    print(f"config1: {[r['n_rows'] for r in meta['runs']]} rows, {time.time() - t0:.1f}s")


CASES = {
    "planted_ngg": case_planted_ngg,
    "mixed_pam": case_mixed_pam,
    "n_gate": case_n_gate,
    "overflow": case_overflow,
    "repeats": case_repeats,
    "many_guides": case_many_guides,
    "seam_5prime": case_seam_5prime,
    "convert": case_convert,
    "config1": case_config1,
    "sacas9_21nt": case_sacas9_21nt,
}

if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--only", nargs="*")
    ap.add_argument("--reference", help="reference checkout (sets BGO_REFERENCE_ROOT)")
    ap.add_argument("--workers", type=int, default=1,
                    help="processes the shim runs each kernel launch in")
    a = ap.parse_args()
    _refshim.set_workers(a.workers)
    for name, fn in CASES.items():
        if a.only and name not in a.only:
            continue
        fn()
