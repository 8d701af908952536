"""Editable-base window logic (beguidedoff/base_editing.py:9-91)."""
from typing import List, Tuple

_TARGET = {"CBE": "C", "ABE": "A", "CGE": "C"}
TARGET_2BIT = {"CBE": 1, "ABE": 0, "CGE": 1}


def editable_base_in_window(offtarget_seq: str, editor_type: str, edit_window_start: int,
                            edit_window_end: int) -> List[int]:
    seq = offtarget_seq.upper()
    tb = _TARGET.get(editor_type)
    if tb is None:
        raise ValueError(f"Unknown editor_type: {editor_type}")
    return [i + 1 for i in range(edit_window_start - 1, edit_window_end)
            if i < len(seq) and seq[i] == tb]


def get_trinucleotide_contexts(seq: str, positions: List[int]) -> List[str]:
    seq = seq.upper()
    out = []
    for pos in positions:
        i = pos - 1
        left = seq[i - 1] if i > 0 else "N"
        right = seq[i + 1] if i < len(seq) - 1 else "N"
        out.append(left + seq[i] + right)
    return out


def has_editable_base(offtarget_seq: str, editor_type: str, edit_window_start: int,
                      edit_window_end: int) -> bool:
    return bool(editable_base_in_window(offtarget_seq, editor_type, edit_window_start,
                                        edit_window_end))


def read_profiles(profiles_path: str) -> List[dict]:
    """Rows of a base_editor_profiles.tsv as dicts (tab separated, header)."""
    with open(profiles_path) as fh:
        lines = [ln.rstrip("\n") for ln in fh if ln.strip()]
    cols = lines[0].split("\t")
    return [dict(zip(cols, ln.split("\t"))) for ln in lines[1:]]


def get_edit_window_from_profile(base_editor: str, profiles_path: str) -> Tuple[int, int, str]:
    rows = read_profiles(profiles_path)
    required = {"name", "general_edit_start", "general_edit_end", "pam"}
    missing = required - set(rows[0] if rows else {})
    if missing:
        raise ValueError(f"Base editor profiles file {profiles_path} is missing required "
                         f"columns: {sorted(missing)}")
    for r in rows:
        if r["name"] == base_editor:
            return int(r["general_edit_start"]), int(r["general_edit_end"]), str(r["pam"])
    names = sorted(r["name"] for r in rows[:5])
    more = "..." if len(rows) > 5 else ""
    raise ValueError(f"Unknown base editor '{base_editor}' in {profiles_path}. "
                     f"Available profiles include: {', '.join(names)}{more}")
