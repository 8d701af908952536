"""API dataclasses (same fields as beguidedoff/types.py:7-49)."""
from dataclasses import dataclass, field
from typing import List, Optional


@dataclass(frozen=True)
class GuideInput:
    """Input specification for one guide RNA (beguidedoff/types.py:7-21)."""

    guide_id: str
    guide_seq: str                # 20 nt, ACGT
    pam: str                      # 1-6 IUPAC characters
    pam_position: str             # only "3prime" is searched
    edit_window_start: int        # 1-based, from the 5' end of the guide
    edit_window_end: int          # 1-based, inclusive
    editor_type: str              # "CBE", "ABE" or "CGE"
    on_target_chrom: Optional[str] = None
    on_target_pos: Optional[int] = None    # 1-based (rightmost for the - strand)
    on_target_strand: Optional[str] = None
    base_editor: Optional[str] = None


@dataclass
class OffTarget:
    """One off-target hit (beguidedoff/types.py:24-41)."""

    chromosome: str
    position: int                 # 1-based; rightmost position on the - strand
    strand: str
    offtarget_seq: str
    genomic_pam: str
    input_pam: str
    guide_seq: str
    base_editor: str
    n_mismatches: int
    mismatch_positions: List[int]
    score: float
    editable_bases: List[int]
    base_edit_context: List[str]


@dataclass
class GuideResult:
    """Results for one guide RNA (beguidedoff/types.py:44-49)."""

    guide_id: str
    total_offtargets: int
    top_offtargets: List[OffTarget] = field(default_factory=list)
