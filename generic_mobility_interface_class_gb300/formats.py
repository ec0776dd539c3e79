"""The reference's text output and checkpoint formats.

* ``.backup`` (cilia_sim_main.cpp:370-381, read back at :29-77): one line,
  the number of completed steps, then every state value of every swimmer in
  ``std::scientific`` with ``setprecision(10)``.  The value order is the one
  of ``gmi_sim_export_backup`` (filament.cpp:1595-1650, rigid_body.cpp:408-432).
* ``.dat`` time series, one line appended per saved step:
  ``_seg_states.dat`` (segment quaternions) and ``_body_states.dat`` (body
  x then q) start with nt + 1 (cilia_sim_main.cpp:346-366, swimmer.cpp:902-912);
  ``_seg_vels.dat``, ``_seg_forces.dat``, ``_body_vels.dat`` and
  ``_blob_forces.dat`` start with nt (mobility_solver.cpp:1775-1895); the wall
  configuration writes no body velocity or blob force files.
"""
from __future__ import annotations

import numpy as np

DIGITS = 10  # std::setprecision(10) with std::scientific


def backup_count(nswim: int, nfil: int, nseg: int) -> int:
    """Values in a backup: per swimmer 19 body values and 9 + 28 NSEG per
    filament (cilia_sim_main.cpp:39-51)."""
    return nswim * (19 + nfil * (9 + 28 * nseg))


def _fmt(values, digits: int) -> str:
    return " ".join(f"{v:.{digits}e}" for v in np.asarray(values, dtype=np.float64).ravel())


def format_backup(nt_completed: int, values, digits: int = DIGITS) -> str:
    """The text of a .backup file: the completed step count, the values, a
    newline (the reference leaves a trailing space before it)."""
    return f"{int(nt_completed)} " + _fmt(values, digits) + " \n"


def parse_backup(text: str):
    """(completed steps, values) from the text of a .backup file."""
    tok = text.split()
    if not tok:
        raise ValueError("empty backup")
    return int(tok[0]), np.array(tok[1:], dtype=np.float64)


def write_backup(path: str, nt_completed: int, values, digits: int = DIGITS) -> None:
    with open(path, "w") as fh:
        fh.write(format_backup(nt_completed, values, digits))


def read_backup(path: str):
    with open(path) as fh:
        return parse_backup(fh.read())


def dat_line(step_label: int, values, digits: int = DIGITS) -> str:
    return f"{int(step_label)} " + _fmt(values, digits) + " \n"


def append_dat(path: str, step_label: int, values, digits: int = DIGITS) -> None:
    with open(path, "a") as fh:
        fh.write(dat_line(step_label, values, digits))


def write_step_data(prefix: str, nt: int, seg_q, body_x, body_q, seg_v, seg_f, body_v=None, blob_f=None,
                    digits: int = DIGITS) -> None:
    """Append one saved step to the reference's six .dat files under prefix
    (pass body_v = blob_f = None for the wall)."""
    body = np.hstack([np.asarray(body_x).reshape(-1, 3), np.asarray(body_q).reshape(-1, 4)])
    append_dat(prefix + "_seg_states.dat", nt + 1, seg_q, digits)
    append_dat(prefix + "_body_states.dat", nt + 1, body, digits)
    if body_v is not None:
        append_dat(prefix + "_body_vels.dat", nt, body_v, digits)
    if blob_f is not None:
        append_dat(prefix + "_blob_forces.dat", nt, blob_f, digits)
    append_dat(prefix + "_seg_vels.dat", nt, seg_v, digits)
    append_dat(prefix + "_seg_forces.dat", nt, seg_f, digits)


def read_dat(path: str):
    """(step labels, rows) of a .dat time series."""
    labels, rows = [], []
    with open(path) as fh:
        for ln in fh:
            tok = ln.split()
            if tok:
                labels.append(int(float(tok[0])))
                rows.append(np.array(tok[1:], dtype=np.float64))
    return np.array(labels), (np.stack(rows) if rows else np.zeros((0, 0)))


__all__ = ["backup_count", "format_backup", "parse_backup", "write_backup", "read_backup", "dat_line",
           "append_dat", "write_step_data", "read_dat", "DIGITS"]
