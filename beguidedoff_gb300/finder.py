"""Extensive-mode finder: the drop-in for beguidedoff/finder.py:256-679.

Same constructor, ``search()`` signature, output columns, row order, sorting,
error types and log messages as the reference.  The genome strands stay on the
GPU (``bgo_genome_create``); one device scan covers every scan key and both
strands (``bgo_scan_launch``), and the exact hit keys come back sorted.  All
host post-processing is vectorised NumPy over the hit arrays instead of the
reference's per-hit Python loops.

Reference behaviours kept on purpose (each pinned by tests/golden):
  * strand '-' positions map through the reverse-complement array per
    chromosome (finder.py:43-62); windows straddling chromosome junctions are
    reported as the reference reports them, including a chromosome index of -1
    (Python's last element) for negative leftmost positions;
  * on-target exclusion on (chromosome index, local leftmost, strand)
    (finder.py:208-218); ``ot_sequence`` / ``ot_pam`` decoded from the scanned
    strand array, so an N reads as A on '+' and T on '-' (:221-234);
  * mismatch positions from guide vs decoded window, so N-corrected positions
    are counted in ``n_mismatches`` but not listed (:435-437);
  * ``include_non_editable`` is ignored; ``return_all`` decides (:508);
  * per-strand hit limits of the re-scan escalation (:568-638): a scan key
    whose hits on a strand exceed ``max_results_per_guide`` keeps that many
    (here: the genome-order prefix) and a warning gives the exact count.
"""
import logging
import threading
import time
from collections import defaultdict
from pathlib import Path
from typing import Dict, List, Optional, Sequence, Tuple

import numpy as np

from . import _native
from .base_editing import TARGET_2BIT
from .encoding import encode_bytes, encode_dna, encode_guide_64bit, extract_windows
from .genome_converter import load_genome
from .io import load_guides_from_tsv
from .pam import encode_pam_mask
from .scoring import scores_of_masks
from .table import COLUMNS, Table, concat, pandas_available
from .types import GuideInput

_LOGGER = logging.getLogger("beguidedoff")

_DEFAULT_RESULTS_PER_GUIDE = 10240
_MAX_RESULTS_PER_GUIDE = 2_621_440
_DECODE = np.array(list("ACGT"))
# up to this many chromosomes the device order key holds the name rank exactly
_EXACT_ORDER_CHROMS = 1024
_PROFILES = str(Path(__file__).resolve().parent / "base_editor_profiles.tsv")


def _device_index(device) -> int:
    if device is None:
        try:
            n = _native.device_count()
        except _native.NativeLibraryMissing:
            raise
        if n == 0:
            raise RuntimeError("Extensive mode requires a CUDA GPU (no CUDA device is visible). "
                               "Use the fast CPU mode instead: "
                               "`beguidedoff(mode='fast', index_path=...)`.")
        return 0
    spec = str(device)
    if not spec.startswith("cuda"):
        raise RuntimeError(f"Extensive mode requires a CUDA GPU (device '{spec}'). "
                           "Use the fast CPU mode instead: "
                           "`beguidedoff(mode='fast', index_path=...)`.")
    return int(spec.split(":")[1]) if ":" in spec else 0


def prepare_n_masks(genome: dict) -> Tuple[Optional[np.ndarray], Optional[np.ndarray]]:
    """Little-bit-order N masks for the forward and reverse-complement arrays
    (finder.py:310-345), padded by 16 bytes; (None, None) without any N."""
    packed_big = genome.get("n_mask")
    total_bp = int(genome["total_bp"])
    if packed_big is None or np.asarray(packed_big).size == 0:
        return None, None
    bits = np.unpackbits(np.asarray(packed_big, dtype=np.uint8), bitorder="big", count=total_bp)
    if not bits.any():
        return None, None
    fwd = np.pad(np.packbits(bits, bitorder="little"), (0, 16))
    rc_bits = np.empty_like(bits)
    for off, ln in zip(np.asarray(genome["chrom_offsets"]), np.asarray(genome["chrom_lengths"])):
        off, ln = int(off), int(ln)
        rc_bits[off:off + ln] = bits[off:off + ln][::-1]
    rc = np.pad(np.packbits(rc_bits, bitorder="little"), (0, 16))
    return fwd, rc


_ASCII = np.frombuffer(b"ACGT", dtype=np.uint8)
_GUIDE_SHIFTS = np.arange(0, 40, 2, dtype=np.uint64)


def _decode_strings(seq: np.ndarray, pam: np.ndarray, plen: np.ndarray):
    """Window and PAM strings of decoded 2-bit rows (object arrays of str)."""
    n = seq.shape[0]
    if n == 0:
        return np.zeros(0, dtype=object), np.zeros(0, dtype=object)
    # one decode of all the bytes, then slices (cheaper than a numpy string
    # dtype round trip at the sizes a table has)
    sr = _ASCII[seq].tobytes().decode("ascii")
    pr = _ASCII[pam].tobytes().decode("ascii")
    s = np.array([sr[20 * i:20 * i + 20] for i in range(n)] + [None], dtype=object)[:-1]
    p = np.array([pr[6 * i:6 * i + k] for i, k in enumerate(plen.tolist())] + [None],
                 dtype=object)[:-1]
    return s, p


# Output strings and rounded scores are functions of the 20-bit mismatch mask
# alone, so they are built once per mask and reused across searches.
_MM_POSITIONS: Dict[int, str] = {}
_ROUND6: Dict[float, float] = {}


def _mismatch_positions(m: int) -> str:
    """1-based mismatch positions of a mask, "1,5" (encoding.py:94-102)."""
    out = _MM_POSITIONS.get(m)
    if out is None:
        out = ",".join(str(i + 1) for i in range(20) if (m >> i) & 1)
        _MM_POSITIONS[m] = out
    return out


def _round6(v: float) -> float:
    """The table's score rounding (round(score, 6), io.py:155-180)."""
    out = _ROUND6.get(v)
    if out is None:
        out = round(v, 6)
        if len(_ROUND6) < (1 << 21):
            _ROUND6[v] = out
    return out


def _guide_bases(seqs: List[str]) -> np.ndarray:
    """[n, 20] 2-bit bases of guide strings (shorter ones zero-padded)."""
    n = len(seqs)
    if n and all(len(q) == 20 for q in seqs):
        return encode_bytes("".join(seqs).encode("ascii", errors="replace")).reshape(n, 20)
    gb = np.zeros((n, 20), dtype=np.uint8)
    for i, q in enumerate(seqs):
        enc = encode_dna(q)[:20]
        gb[i, :enc.size] = enc
    return gb


def _per_unique(values: np.ndarray, fn, cache: Optional[dict] = None) -> np.ndarray:
    """fn applied once per distinct value, spread back (an object array).
    ``cache`` is fn's memo: small arrays are mapped through it in one pass,
    calling fn only for values it does not hold yet."""
    if values.size == 0:
        return np.zeros(0, dtype=object)
    if values.size <= 4096:  # fn is memoised: a direct pass is cheaper than unique
        vals = values.tolist()
        out = list(map(cache.get, vals)) if cache is not None else [None] * len(vals)
        if None in out:
            out = [fn(v) if o is None else o for o, v in zip(out, vals)]
        return np.array(out + [None], dtype=object)[:-1]
    uniq, inv = np.unique(values, return_inverse=True)
    mapped = np.array([fn(v) for v in uniq.tolist()] + [None], dtype=object)[:-1]
    return mapped[inv.ravel()]


def window_cols(g) -> List[int]:
    """Guide positions of the edit window as Python indexes a 20-nt string:
    range(start - 1, end) below 20, negative indexes from the end
    (beguidedoff/base_editing.py:8-27 slices the decoded window this way)."""
    cols = [i if i >= 0 else 20 + i
            for i in range(g.edit_window_start - 1, g.edit_window_end) if i < 20]
    if any(c < 0 for c in cols):
        raise IndexError("string index out of range")
    return cols


def epilogue_inputs(pairs, threshold_rank: int = -1, return_all: bool = False
                    ) -> Optional[np.ndarray]:
    """Device epilogue rows (bgo_input_row) for (plan row, GuideInput,
    (on-target chromosome index, local leftmost, strand) or Nones) triples;
    None if an editor type is unknown (the host path raises its error)."""
    rows = []
    flags = _native.ROW_RETURN_ALL if return_all else 0
    for plan_row, g, ot in pairs:
        tb = TARGET_2BIT.get(g.editor_type)
        if tb is None:
            return None
        mask = 0
        for c in window_cols(g):
            mask |= 1 << c
        has_ot = ot[0] is not None
        rows.append((plan_row, mask, tb, ot[0] if has_ot else -1, ot[1] if has_ot else 0,
                     0 if ot[2] == "+" else 1, threshold_rank, flags, 0))
    return np.array(rows, dtype=_native.INPUT_ROW_DTYPE)


class beguidedoff:
    """GPU brute-force off-target search (extensive mode)."""

    def __init__(self, genome_path: str, max_mismatches: int = 4, scoring_method: str = "CCTOP",
                 device: Optional[str] = None, n_top_offtargets: int = 3,
                 results_per_guide: int = 10240, max_results_per_guide: Optional[int] = None,
                 genome_data: Optional[dict] = None, scan_mode="auto",
                 epilogue: str = "device", scan_tuning: Optional[Sequence[int]] = None):
        if epilogue not in ("device", "host"):
            raise ValueError("epilogue must be 'device' or 'host'")
        self.epilogue = epilogue
        self.genome_path = genome_path
        self.max_mismatches = max_mismatches
        if scoring_method.upper() != "CCTOP":
            raise ValueError("extensive mode only supports scoring_method='CCTOP'")
        self.scoring_method = "CCTOP"
        self.n_top_offtargets = n_top_offtargets
        self.results_per_guide = results_per_guide
        self.max_results_per_guide = max_results_per_guide
        if scan_mode != "auto" and scan_mode not in (0, 1, 2, 3):
            raise ValueError("scan_mode must be 'auto' or 0..3")
        self.scan_mode = scan_mode
        # with a fixed scan_mode: the launch parameters every plan gets
        # (Plan.set_tuning's positional fields); None keeps the defaults
        self.scan_tuning = tuple(scan_tuning) if scan_tuning is not None else None
        self._tuner = None
        self._tuner_lock = threading.Lock()
        self.last_choice = None
        self.last_batch = None
        self.device_index = _device_index(device)
        self.device = f"cuda:{self.device_index}"
        self._init_host(genome_data if genome_data is not None else load_genome(genome_path))
        self._engine = _native.Engine(self.device_index)
        masks = [self._n_mask_fwd, self._n_mask_rc][:len(self._strand_arrays)]
        self._strands = [_native.Strand(a, self.total_bp, m, self.device_index)
                         for a, m in zip(self._strand_arrays, masks)]

    def _init_host(self, genome_data: dict) -> None:
        """Host-side genome tables (no device state)."""
        self.genome_data = g = genome_data
        self.total_bp = int(g["total_bp"])
        self.chrom_names = [str(c) for c in g["chrom_names"]]
        self.chrom_offsets = np.asarray(g["chrom_offsets"], dtype=np.int64)
        self.chrom_lengths = np.asarray(g["chrom_lengths"], dtype=np.int64)
        self._n_mask_fwd, self._n_mask_rc = prepare_n_masks(g)
        self._strand_arrays = [np.ascontiguousarray(g["genome_forward"], dtype=np.uint32)]
        if "genome_rc" in g:
            self._strand_arrays.append(np.ascontiguousarray(g["genome_rc"], dtype=np.uint32))
        order = np.argsort(np.array(self.chrom_names, dtype=object), kind="stable")
        self._chrom_rank = np.empty(len(order), dtype=np.int64)
        self._chrom_rank[order] = np.arange(len(order))

    @classmethod
    def host_only(cls, genome_data: dict, max_mismatches: int = 4, n_top_offtargets: int = 3,
                  results_per_guide: int = 10240, max_results_per_guide: Optional[int] = None):
        """A finder without device state whose ``search_with_keys`` assembles
        the output from externally supplied hit keys (used to test the host
        post-processing without a GPU)."""
        self = cls.__new__(cls)
        self.genome_path = None
        self.max_mismatches = max_mismatches
        self.scoring_method = "CCTOP"
        self.n_top_offtargets = n_top_offtargets
        self.results_per_guide = results_per_guide
        self.max_results_per_guide = max_results_per_guide
        self.scan_mode = 1
        self._tuner = None
        self._tuner_lock = threading.Lock()
        self.last_choice = None
        self.last_batch = None
        self.epilogue = "host"
        self.device_index, self.device = -1, "none"
        self._engine, self._strands = None, []
        self._init_host(genome_data)
        return self

    @property
    def genome_info(self) -> dict:
        return {"build": "unknown", "total_bp": self.total_bp,
                "n_chromosomes": len(self.chrom_names), "chromosomes": self.chrom_names}

    def close(self):
        if getattr(self, "_tuner", None) is not None:
            self._tuner.close()
            self._tuner = None
        for s in getattr(self, "_strands", []):
            s.close()
        self._strands = []
        if getattr(self, "_engine", None) is not None:
            self._engine.close()
            self._engine = None

    # ------------------------------------------------------------------
    def _deduplicate_guides(self, guides: List[GuideInput]):
        """Scan keys (seq, pam, on-target chrom index, local leftmost, strand)
        in first-seen order and the input rows of each (finder.py:361-403)."""
        mapping: Dict[tuple, List[GuideInput]] = defaultdict(list)
        for g in guides:
            ci = lp = st = None
            if g.on_target_chrom and g.on_target_pos is not None:
                ci = next((i for i, n in enumerate(self.chrom_names)
                           if n == g.on_target_chrom), None)
                if ci is not None:
                    if g.on_target_strand is None:
                        raise ValueError(
                            f"Guide {g.guide_id} has on-target chromosome and position but no "
                            f"strand. Please provide on_target_strand ('+' or '-').")
                    window = 20 + len(g.pam)
                    lp = g.on_target_pos - 1 if g.on_target_strand == "+" else \
                        g.on_target_pos - window
                    st = g.on_target_strand
            mapping[(g.guide_seq, g.pam, ci, lp, st)].append(g)
        return list(mapping), mapping

    def _plan(self, plan_seqs: List[str], plan_pams: List[str], engine=None, stream=None):
        n = len(plan_seqs)
        if n and all(len(s) == 20 for s in plan_seqs):
            # every row at once: base i of row r at bits 2 * i
            codes = encode_bytes("".join(plan_seqs).encode("ascii", errors="replace"))
            gv = np.bitwise_or.reduce(codes.reshape(n, 20).astype(np.uint64)
                                      << _GUIDE_SHIFTS[None, :], axis=1)
        else:
            gv = np.array([encode_guide_64bit(encode_dna(s)[:20]) for s in plan_seqs],
                          dtype=np.uint64)
        masks = {p: encode_pam_mask(p) for p in set(plan_pams)}
        pm = np.stack([masks[p] for p in plan_pams]) if n else np.zeros((0, 6), dtype=np.uint8)
        pl = np.array([len(p) for p in plan_pams], dtype=np.uint8)
        p3 = np.ones(n, dtype=np.uint8)
        return _native.Plan(engine or self._engine, gv, pm, pl, p3, stream)

    def _mode_for(self, plan, plan_pams: List[str], max_mismatches: Optional[int] = None) -> int:
        """The scan mode to run: the constructor's, or the autotuner's choice
        (which also sets the plan's launch tuning)."""
        if self.scan_mode != "auto":
            if self.scan_tuning is not None:
                plan.set_tuning(*self.scan_tuning)
            return int(self.scan_mode)
        k = self.max_mismatches if max_mismatches is None else max_mismatches
        with self._tuner_lock:
            if self._tuner is None:
                from .autotune import Autotuner

                masks = [self._n_mask_fwd, self._n_mask_rc][:len(self._strand_arrays)]
                self._tuner = Autotuner(self._engine, self._strand_arrays, masks, self.total_bp,
                                        self.device_index,
                                        coarse=getattr(self, "tune_per_k", False))
            self.last_choice = self._tuner.choose(plan, plan_pams, k)
            return self.last_choice.mode

    def _scan(self, plan_seqs: List[str], plan_pams: List[str]) -> np.ndarray:
        """Device scan of both strands; sorted hit keys."""
        plan = self._plan(plan_seqs, plan_pams)
        try:
            mode = self._mode_for(plan, plan_pams)
            ne = [0, 3][:len(self._strands)]
            return self._engine.scan(plan, self._strands, ne, self.max_mismatches, mode=mode)
        finally:
            plan.close()

    def _prepare(self, guides: List[GuideInput]):
        """Checks of the reference's search() and the dedup to scan keys."""
        if not guides:
            raise ValueError("No guides provided")
        for g in guides:
            if g.pam_position.lower() != "3prime":
                raise ValueError(f"Guide {g.guide_id} has pam_position '{g.pam_position}'. "
                                 f"Only 3prime PAM is supported.")
        return self._deduplicate_guides(guides)

    def _run_batch(self, reqs: List[dict], max_mismatches: int, engine=None, stream=None,
                   log=None, info: Optional[dict] = None) -> List[object]:
        """One plan, one scan and one device epilogue for several searches with
        the same max_mismatches.  Each request dict holds ``keys``,
        ``mapping``, ``guides``, ``return_all`` and ``count_score_threshold``;
        its input rows, options and assembly stay its own, so its table is the
        one search() returns for it alone.  Returns a table or an exception
        per request."""
        from .scoring import score_ranks, threshold_rank

        eng = engine or self._engine
        log = log if log is not None else _LOGGER
        plan_index: Dict[tuple, int] = {}
        for r in reqs:
            r["key_plan"] = np.array([plan_index.setdefault((k[0], k[1]), len(plan_index))
                                      for k in r["keys"]], dtype=np.int64)
        plan_items = list(plan_index)
        pams = [p for _, p in plan_items]
        t0 = time.perf_counter()
        plan = self._plan([s for s, _ in plan_items], pams, eng, stream)
        try:
            mode = self._mode_for(plan, pams, max_mismatches)
            t1 = time.perf_counter()
            ne = [0, 3][:len(self._strands)]
            eng.launch(plan, self._strands, ne, max_mismatches, mode, stream)
            # the epilogue's input rows are built on the host while the scan runs
            parts, owners, spans, errs = [], [], [], []
            n_rows = 0
            for r in reqs:
                pairs = [(int(r["key_plan"][ki]), g, key[2:]) for ki, key in enumerate(r["keys"])
                         for g in r["mapping"][key]]
                try:
                    rows = epilogue_inputs(pairs, threshold_rank(r["count_score_threshold"]),
                                           r["return_all"])
                except Exception as exc:  # the host path raises the same error
                    rows = None
                    errs.append(exc)
                else:
                    errs.append(None)
                if rows is None:   # unknown editor or bad window: host path
                    spans.append(None)
                    owners.append(None)
                    continue
                spans.append((n_rows, len(pairs)))
                n_rows += len(pairs)
                parts.append(rows)
                owners.append([g.guide_id for _, g, _ in pairs])
            # every hit in the buffer: an overflowing scan rescans only the
            # granules whose keys did not fit
            n = eng.complete(plan, self._strands, ne, max_mismatches, mode, stream)
            t2 = time.perf_counter()
            # this batch's own record (batches of several serving slots run
            # concurrently; last_batch only ever receives a finished record)
            stats = {"hits": n, "plan_rows": len(plan_items), "mode": mode,
                     "plan_s": t1 - t0, "scan_s": t2 - t1}
            if info is not None:
                info.update(stats)
            full = None
            if parts:
                rank_table, _ = score_ranks()
                below, groups, counts, recs = eng.epilogue(
                    plan, self._strands, np.concatenate(parts), self.chrom_offsets,
                    self.chrom_lengths, self._chrom_rank, rank_table, self.n_top_offtargets,
                    stream)
                rec_off = np.concatenate([[0], np.cumsum(counts)])
            t3 = time.perf_counter()
            out = []
            for i, r in enumerate(reqs):
                try:
                    if errs[i] is not None:
                        raise errs[i]
                    pre = None
                    if spans[i] is not None:
                        counts_k = groups[r["key_plan"]]
                        limit = self._limits(counts_k, r["keys"], log)
                        if not (counts_k.max(axis=1) > limit).any():
                            r0, nr = spans[i]
                            below_by_id: Dict[str, int] = defaultdict(int)
                            if r["count_score_threshold"] is not None:
                                for gid, b in zip(owners[i], below[r0:r0 + nr].tolist()):
                                    below_by_id[gid] += b
                            pre = (limit, below_by_id if r["count_score_threshold"] is not None
                                   else None)
                    if pre is not None and len(self.chrom_names) <= _EXACT_ORDER_CHROMS:
                        r0, nr = spans[i]
                        out.append(self._table_from_records(
                            recs[rec_off[r0]:rec_off[r0 + nr]], r0, owners[i], r["guides"],
                            plan_items, r["return_all"], pre[1]))
                        continue
                    if pre is None:
                        # a strand hit limit is reached (the genome-order prefix
                        # of every strand is needed) or an editor type is unknown
                        if full is None:
                            _, full = eng.collect(stream)
                        hit_keys = full
                    else:
                        r0, nr = spans[i]
                        hit_keys = np.unique(recs["key"][rec_off[r0]:rec_off[r0 + nr]])
                    out.append(self._assemble(hit_keys, r["keys"], r["key_plan"], plan_items,
                                              r["mapping"], r["guides"], r["return_all"],
                                              r["count_score_threshold"], log, precomputed=pre))
                except Exception as exc:  # reported to that request only
                    out.append(exc)
            stats["epilogue_s"] = (t3 - t2) if parts else 0.0
            stats["assemble_s"] = time.perf_counter() - (t3 if parts else t2)
            if info is not None:
                info.update(stats)
            self.last_batch = stats
            return out
        finally:
            plan.close()

    def _limits(self, counts2: np.ndarray, keys, log) -> np.ndarray:
        """Per scan key the per-strand number of hits kept, with the warnings
        of the reference's overflow re-scan loop (finder.py:568-638)."""
        cap = (self.max_results_per_guide if self.max_results_per_guide is not None
               else _MAX_RESULTS_PER_GUIDE)
        mx = counts2.max(axis=1) if counts2.size else np.zeros(0, dtype=np.int64)
        limit = np.full(len(keys), self.results_per_guide, dtype=np.int64)
        pending = np.nonzero(mx > self.results_per_guide)[0]
        rpg = self.results_per_guide
        while pending.size:
            if rpg >= cap:
                for i in sorted(pending.tolist(), key=lambda j: keys[j][0]):
                    log.warning(
                        "Truncated off-target enumeration for guide %s (PAM=%s): %d raw "
                        "genome-wide hits exceed the per-strand buffer of %d; keeping the "
                        "first %d (genome order). The off-target count for this guide is a "
                        "lower bound.", keys[i][0], keys[i][1], int(counts2[i].sum()), rpg,
                        int(np.minimum(counts2[i], rpg).sum()))
                break
            rpg = min(rpg * 16, cap)
            if log is not None:
                names = ", ".join(sorted({keys[i][0] for i in pending.tolist()})[:5])
                log.warning("Hit buffer overflow for %d guide(s) at results_per_guide=%s "
                            "(e.g. %s); re-scanning them with results_per_guide=%d.",
                            pending.size, self.results_per_guide, names, rpg)
            limit[pending] = rpg
            pending = pending[mx[pending] > rpg]
        return limit

    # ------------------------------------------------------------------
    def search(self, input_file: Optional[str] = None, guides: Optional[List[GuideInput]] = None,
               return_all: bool = False, count_score_threshold: Optional[float] = None,
               output_file: Optional[str] = None, include_non_editable: bool = False,
               presets_path: Optional[str] = None, verbose: bool = True,
               logger: Optional[logging.Logger] = None):
        if (input_file is None) == (guides is None):
            raise ValueError("Exactly one of input_file or guides must be provided")
        if input_file is not None:
            guides = load_guides_from_tsv(input_file, presets_path=presets_path or _PROFILES)
        log = logger if logger is not None else _LOGGER
        t_prep = time.perf_counter()
        keys, mapping = self._prepare(guides)
        t_prep = time.perf_counter() - t_prep
        if verbose:
            log.info("Guides after deduplication: %d (from %d input rows)", len(keys),
                     len(guides))
            log.info("Running GPU search on %s ...", self.device)
        if self.epilogue == "device":
            table = self._run_batch([{"keys": keys, "mapping": mapping, "guides": guides,
                                      "return_all": return_all,
                                      "count_score_threshold": count_score_threshold}],
                                    self.max_mismatches, log=log)[0]
            if isinstance(table, Exception):
                raise table
            if self.last_batch is not None:
                self.last_batch["prepare_s"] = t_prep
        else:
            # one plan row per distinct (seq, pam); scan keys that differ only
            # in their on-target share it
            plan_index: Dict[tuple, int] = {}
            key_plan = np.empty(len(keys), dtype=np.int64)
            for i, k in enumerate(keys):
                key_plan[i] = plan_index.setdefault((k[0], k[1]), len(plan_index))
            plan_items = list(plan_index)
            hit_keys = self._scan([s for s, _ in plan_items], [p for _, p in plan_items])
            table = self._assemble(hit_keys, keys, key_plan, plan_items, mapping, guides,
                                   return_all, count_score_threshold, log)
        if output_file:
            table.to_csv(output_file, sep="\t", index=False)
            if verbose:
                log.info("Wrote results to %s", output_file)
        return table

    # ------------------------------------------------------------------
    def _chrom_name_array(self) -> np.ndarray:
        """The chromosome names as an object array (built once)."""
        arr = getattr(self, "_chrom_names_arr", None)
        if arr is None or len(arr) != len(self.chrom_names):
            arr = np.array(list(self.chrom_names) + [None], dtype=object)[:-1]
            self._chrom_names_arr = arr
        return arr

    def _table_from_records(self, recs, row0, owners, guides, plan_items, return_all,
                            below_by_id):
        """Output table straight from the device epilogue's records: each
        input row's hits among its n_top smallest order keys (score rank,
        chromosome name rank, local report position, strand - the order of
        beguidedoff/finder.py:545-566).  Per guide id the rows' records are
        merged in input-row order, sorted by order key and cut to n_top (all
        with return_all); every input row of that id then gets the id's
        table, with its own base editor, as in _assemble."""
        n_top = self.n_top_offtargets
        local = recs["input_row"].astype(np.int64) - row0
        gid_code: Dict[str, int] = {}
        row_code = np.array([gid_code.setdefault(gid, len(gid_code)) for gid in owners],
                            dtype=np.int64)
        rec_code = row_code[local] if local.size else np.zeros(0, dtype=np.int64)
        # ties (possible only between identical hits of rows sharing a plan
        # row) keep _assemble's order: input row, then hit key
        order = np.lexsort((recs["key"], local, recs["order"], rec_code))
        codes_sorted = rec_code[order]
        first = np.searchsorted(codes_sorted, codes_sorted, side="left")
        rank = np.arange(order.size) - first
        keep = order if return_all else order[rank < n_top]
        kcode = rec_code[keep]
        # per guide id: its kept records, in order
        bounds = np.searchsorted(kcode, np.arange(len(gid_code) + 1), side="left")
        # decode the kept hits (vectorised)
        row, slot, pos, mm = _native.split_keys(recs["key"][keep])
        n = keep.size
        seq = np.zeros((n, 20), dtype=np.uint8)
        pam = np.zeros((n, 6), dtype=np.uint8)
        for st in range(len(self._strand_arrays)):
            sel = np.nonzero(slot == st)[0]
            if sel.size:
                arr = self._strand_arrays[st]
                seq[sel] = extract_windows(arr, pos[sel], 20)
                pam[sel] = extract_windows(arr, pos[sel] + 20, 6)
        plan_seq = np.array([q for q, _ in plan_items] + [None], dtype=object)[:-1]
        plen = np.array([len(pm) for _, pm in plan_items], dtype=np.int64)[row]
        gb = _guide_bases([g for g, _ in plan_items])
        weights = np.int64(1) << np.arange(20, dtype=np.int64)
        mmask = ((seq != gb[row]).astype(np.int64) * weights[None, :]).sum(1) if n else \
            np.zeros(0, dtype=np.int64)
        score = scores_of_masks(mmask)
        offsets, lengths = self.chrom_offsets, self.chrom_lengths
        window = 20 + plen
        leftmost = pos.copy()
        minus = slot == 1
        if minus.any():
            ci = np.searchsorted(offsets, pos[minus], side="right") - 1
            leftmost[minus] = offsets[ci] + (lengths[ci] - (pos[minus] - offsets[ci]) - window[minus])
        report = np.where(minus, leftmost + window - 1, pos)
        rep_ci = np.searchsorted(offsets, report, side="right") - 1
        rep_local = report - offsets[rep_ci]
        # one block per input guide row, in input order: the id's kept records
        codes = np.array([gid_code.get(g.guide_id, -1) for g in guides], dtype=np.int64)
        cc = np.maximum(codes, 0)
        sizes = np.where(codes >= 0, bounds[cc + 1] - bounds[cc], 0)
        rows_in = np.nonzero(sizes)[0]
        if rows_in.size == 0:
            if pandas_available():
                import pandas as pd

                return pd.DataFrame()
            return Table()
        sizes = sizes[rows_in]
        starts = bounds[cc[rows_in]]
        ends = np.cumsum(sizes)
        within = np.arange(int(ends[-1]), dtype=np.int64) - np.repeat(ends - sizes, sizes)
        idx = np.repeat(starts, sizes) + within
        bid = below_by_id or {}
        editors = [guides[i].base_editor or "" for i in rows_in.tolist()]
        below = [bid.get(guides[i].guide_id, 0) for i in rows_in.tolist()]
        seq_s, pam_s = _decode_strings(seq[idx], pam[idx], plen[idx])
        mpos = _per_unique(mmask[idx], _mismatch_positions, _MM_POSITIONS)
        cols = {
            "guide_rna_sequence": plan_seq[row[idx]],
            "base_editor": np.repeat(np.array(editors, dtype=object), sizes),
            "ot_rank": within + 1,
            "ot_chromosome": self._chrom_name_array()[rep_ci[idx]],
            "ot_position": (rep_local[idx] + 1).astype(np.int64),
            "ot_strand": np.where(slot[idx] == 1, "-", "+").astype(object),
            "ot_sequence": np.array(seq_s, dtype=object),
            "ot_pam": np.array(pam_s, dtype=object),
            "n_mismatches": mm[idx].astype(np.int64),
            "mismatch_positions": np.array(mpos, dtype=object),
            "score": _per_unique(score[idx], _round6, _ROUND6).astype(np.float64),
            "n_offtargets_below_threshold": np.repeat(np.array(below, dtype=np.int64), sizes),
        }
        t = Table(cols, COLUMNS)
        return t.to_pandas() if pandas_available() else t

    def _assemble(self, hit_keys, keys, key_plan, plan_items, mapping, guides, return_all,
                  count_score_threshold, log, precomputed=None):
        """Output table from sorted hit keys.  ``precomputed`` = (per-key
        strand limits, below-threshold counts by guide id or None) when the
        keys are only the device epilogue's top-N candidates: no limit is
        reached then, and the counts cover every hit."""
        row, slot, pos, mm = _native.split_keys(hit_keys)
        n_plan = len(plan_items)
        if precomputed is None:
            counts2 = np.zeros((n_plan, 2), dtype=np.int64)
            np.add.at(counts2, (row, slot), 1)
            limit = self._limits(counts2[key_plan], keys, log)
        else:
            limit = precomputed[0]
        offsets, lengths = self.chrom_offsets, self.chrom_lengths
        # keys are sorted by (row, strand, position): ranges per row, and the
        # rank of each hit inside its (row, strand) group
        r_lo = np.searchsorted(row, np.arange(n_plan), side="left")
        r_hi = np.searchsorted(row, np.arange(n_plan), side="right")
        grp = row * 2 + slot
        rank = np.arange(grp.size) - np.searchsorted(grp, grp, side="left")
        plen_plan = np.array([len(p) for _, p in plan_items], dtype=np.int64)
        # decode windows and PAMs from the scanned strand arrays
        seq = np.zeros((grp.size, 20), dtype=np.uint8)
        pam = np.zeros((grp.size, 6), dtype=np.uint8)
        for s in range(len(self._strand_arrays)):
            sel = np.nonzero(slot == s)[0]
            if sel.size:
                arr = self._strand_arrays[s]
                seq[sel] = extract_windows(arr, pos[sel], 20)
                pam[sel] = extract_windows(arr, pos[sel] + 20, 6)
        plen = plen_plan[row]
        window = 20 + plen
        leftmost = pos.copy()
        minus = slot == 1
        if minus.any():
            ci = np.searchsorted(offsets, pos[minus], side="right") - 1
            local_rc = pos[minus] - offsets[ci]
            leftmost[minus] = offsets[ci] + (lengths[ci] - local_rc - window[minus])
        report = np.where(minus, leftmost + window - 1, pos)
        rep_ci = np.searchsorted(offsets, report, side="right") - 1
        rep_local = report - offsets[rep_ci]
        # leftmost as (chromosome index, local) for the on-target test; a
        # negative leftmost gives index -1, which never equals an on-target
        ot_ci_hit = np.searchsorted(offsets, leftmost, side="right") - 1
        ot_local_hit = leftmost - offsets[ot_ci_hit]
        # mismatch masks (guide vs decoded window) and exact CCTOP scores
        mmask = np.zeros(grp.size, dtype=np.int64)
        weights = np.int64(1) << np.arange(20, dtype=np.int64)
        for p_i in range(n_plan):
            a, b = r_lo[p_i], r_hi[p_i]
            if a == b:
                continue
            gb = np.zeros(20, dtype=np.uint8)
            enc = encode_dna(plan_items[p_i][0])[:20]
            gb[:enc.size] = enc
            mmask[a:b] = ((seq[a:b] != gb[None, :]).astype(np.int64) * weights[None, :]).sum(1)
        score = scores_of_masks(mmask)
        include_non_editable = return_all
        below: Dict[str, int] = defaultdict(int)
        if precomputed is not None and precomputed[1] is not None:
            below = precomputed[1]
        per_input: Dict[str, List[np.ndarray]] = defaultdict(list)
        for ki, key in enumerate(keys):
            p_i = key_plan[ki]
            sel = np.arange(r_lo[p_i], r_hi[p_i])
            if precomputed is None:
                sel = sel[rank[sel] < limit[ki]]
            if key[2] is not None and sel.size:
                st_code = 0 if key[4] == "+" else 1
                excl = ((ot_ci_hit[sel] == key[2]) & (ot_local_hit[sel] == key[3])
                        & (slot[sel] == st_code))
                sel = sel[~excl]
            for g in mapping[key]:
                tb = TARGET_2BIT.get(g.editor_type)
                if tb is None:
                    raise ValueError(f"Unknown editor_type: {g.editor_type}")
                cols = window_cols(g)
                if cols and sel.size:
                    editable = (seq[sel][:, cols] == tb).any(axis=1)
                else:
                    editable = np.zeros(sel.size, dtype=bool)
                per_input[g.guide_id].append(sel if include_non_editable else sel[editable])
                if count_score_threshold is not None and precomputed is None:
                    below[g.guide_id] += int(
                        (editable & (score[sel] <= count_score_threshold)).sum())
        tables = []
        for g in guides:
            parts = per_input.get(g.guide_id)
            keep = np.concatenate(parts) if parts else np.zeros(0, dtype=np.int64)
            if keep.size == 0:
                continue
            order = np.lexsort((slot[keep], rep_local[keep], self._chrom_rank[rep_ci[keep]],
                                score[keep]))
            keep = keep[order]
            if not return_all:
                keep = keep[:self.n_top_offtargets]
            tables.append(self._table(keep, g, seq, pam, plen, mm, mmask, score, slot, rep_ci,
                                      rep_local, plan_items, row, below.get(g.guide_id, 0)))
        t = concat(tables) if tables else Table()
        if pandas_available():
            import pandas as pd

            return t.to_pandas() if tables else pd.DataFrame()
        return t

    def _table(self, idx, g, seq, pam, plen, mm, mmask, score, slot, rep_ci, rep_local,
               plan_items, row, n_below):
        n = idx.size
        seq_s = ["".join(r) for r in _DECODE[seq[idx]]]
        pam_s = ["".join(r[:k]) for r, k in zip(_DECODE[pam[idx]], plen[idx].tolist())]
        mpos = [_mismatch_positions(m) for m in mmask[idx].tolist()]
        cols = {
            "guide_rna_sequence": np.array([plan_items[r][0] for r in row[idx].tolist()],
                                           dtype=object),
            "base_editor": np.array([g.base_editor or ""] * n, dtype=object),
            "ot_rank": np.arange(1, n + 1, dtype=np.int64),
            "ot_chromosome": np.array([self.chrom_names[c] for c in rep_ci[idx].tolist()],
                                      dtype=object),
            "ot_position": (rep_local[idx] + 1).astype(np.int64),
            "ot_strand": np.where(slot[idx] == 1, "-", "+").astype(object),
            "ot_sequence": np.array(seq_s, dtype=object),
            "ot_pam": np.array(pam_s, dtype=object),
            "n_mismatches": mm[idx].astype(np.int64),
            "mismatch_positions": np.array(mpos, dtype=object),
            "score": np.array([_round6(v) for v in score[idx].tolist()], dtype=np.float64),
            "n_offtargets_below_threshold": np.full(n, n_below, dtype=np.int64),
        }
        return Table(cols, COLUMNS)
