"""Output and resume formats of the reference, and checkpoints of a batch.

Frame and preliminary time-series CSV files are written exactly as the
reference's save_frame / save_prelimframe write them
(simulations/Percolation_FD/multiSPDP.cpp:1493-1643): header line, C++ default
stream formatting of doubles (6 significant digits, `%g`), and the
collision-safe replicate numbering of findMaxRepNo (:1325-1350): if
`<pattern><r>.csv` exists the file becomes `<pattern><max+1>.csv`.  Frames can
be read back as an initial condition (the reference's burn-in restart,
init_burnin_wrapper :625-693 reading CSV columns).

A checkpoint keeps what this integrator needs to resume bit for bit: the
fields at full precision, the step counter (the Philox counter of the next
step) and the instance table (seeds, control parameters).  There is no
generator state to save.
"""
from __future__ import annotations

import json
import os
import re

import numpy as np

FRAME_HEADER_DP = "a_c,  x,  P(x; t) \n"                              # MultiSPDP_constants_1Sp.h:6
FRAME_HEADER_RIETKERK = "a_c,  x,  P(x; t), W(x; t), O(x; t) \n"     # rietkerk_bjork_constants_1Sp.h:6
PRELIM_HEADER_DP = (" a , r, L, t , <<P(x; t)>_x>_r, Var[<P(x; t)>_x]_r, # Surviving Runs P(x; t),"
                    " # Active Sites P(x; t), \n")                     # MultiSPDP_constants_1Sp.h:8-9
STATS_HEADER_DP = (" a , L, t ,  <<Rho(x; t)>_x>_r, Var[<Rho(t)>_x]_r, # Surviving Runs, # Active Sites,"
                   " # Surviving Runs Alt \n")                         # stochasticSPDP.cpp:1406


def fmt(x) -> str:
    """A double as C++ `std::ostream << double` prints it by default (%g, 6 digits)."""
    if isinstance(x, (int, np.integer)):
        return str(int(x))
    v = float(x)
    if v != v:
        return "-nan" if np.signbit(v) else "nan"
    return format(v, "g")


def find_max_rep_no(parendir: str, filename_pattern: str) -> int:
    """Largest replicate number of files named `<pattern><n>.csv` in parendir
    (findMaxRepNo, multiSPDP.cpp:1325-1350); 0 if none."""
    rx = re.compile(re.escape(filename_pattern) + r"(\d+)\.csv")
    best = 0
    for name in os.listdir(parendir):
        m = rx.fullmatch("/" + name)
        if m:
            best = max(best, int(m.group(1)))
    return best


def _target(parendir, filename_pattern, r, overwrite):
    path = parendir + filename_pattern + str(r) + ".csv"
    if os.path.exists(path) and not overwrite:
        path = parendir + filename_pattern + str(find_max_rep_no(parendir, filename_pattern) + 1) + ".csv"
    return path


def save_frame(fields, parendir: str, filename_pattern: str, a: float, r: int, header: str | None = None,
               overwrite: bool = False) -> str:
    """Write one instance's lattice(s): rows `a,i,f0[i],f1[i],...` for every site i."""
    f = np.asarray(fields)
    if f.ndim == 2:
        f = f[None]
    nf = f.shape[0]
    flat = f.reshape(nf, -1)
    if header is None:
        header = FRAME_HEADER_DP if nf == 1 else FRAME_HEADER_RIETKERK
    parts = [header]
    sa = fmt(a)
    cols = [[fmt(v) for v in flat[s]] for s in range(nf)]
    for i in range(flat.shape[1]):
        parts.append(sa + "," + str(i) + "".join("," + cols[s][i] for s in range(nf)) + "\n")
    path = _target(parendir, filename_pattern, r, overwrite)
    with open(path, "w", newline="") as fh:
        fh.write("".join(parts))
    return path


def save_prelimframe(rows, parendir: str, filename_pattern: str, a: float, r: int, L: int,
                     header: str = PRELIM_HEADER_DP, overwrite: bool = False) -> str:
    """Write a preliminary time series: rows `a,r+1,L,t,` then for each species
    `mean,var,#surviving,#active,` (save_prelimframe, multiSPDP.cpp:1493-1546);
    rows[i] = [t, mean, var, surv, active, (4 more per further species)]."""
    rows = np.asarray(rows, dtype=np.float64)
    nsp = (rows.shape[1] - 1) // 4
    parts = [header]
    head = fmt(a) + "," + str(r + 1) + "," + str(L) + ","
    for row in rows:
        s = head + fmt(row[0]) + ","
        for k in range(nsp):
            s += "".join(fmt(row[4 * k + j]) + "," for j in range(1, 5))
        parts.append(s + "\n")
    path = _target(parendir, filename_pattern, r, overwrite)
    with open(path, "w", newline="") as fh:
        fh.write("".join(parts))
    return path


def save_stats(rows, path: str, header: str = STATS_HEADER_DP) -> str:
    """The sweep's final table {a, L, t, <<rho>_x>_r, Var, #surv, #active, surv-alt}
    (critical_exp_delta, stochasticSPDP.cpp:1396-1421)."""
    with open(path, "w", newline="") as fh:
        fh.write(header)
        for row in np.asarray(rows):
            fh.write(",".join(fmt(v) for v in row) + "\n")
    return path


def read_frame(path: str, L: int, nf: int | None = None) -> np.ndarray:
    """Read a frame CSV back as fields (nf, L, L) (or (L, L) for one field):
    the burn-in initial condition.  Values carry the file's 6 significant digits."""
    with open(path) as fh:
        fh.readline()
        data = np.loadtxt(fh, delimiter=",", ndmin=2)
    vals = data[:, 2:]
    if nf is None:
        nf = vals.shape[1]
    out = vals[:, :nf].T.reshape(nf, L, L)
    return out[0] if nf == 1 else out


def save_checkpoint(batch, path: str) -> None:
    """Fields (full precision), step counter and instance table of a Batch."""
    inst = batch.inst
    meta = {"step": batch.step, "precision": batch.precision, "nf": batch.nf,
            "instances": [[int(i.L), int(i.seed), float(i.a), float(i.a_step)] for i in inst]}
    np.savez(path, fields=batch.download_packed(), meta=np.frombuffer(json.dumps(meta).encode(), np.uint8))


def load_checkpoint(batch, path: str) -> int:
    """Restore fields and step counter into a Batch built with the same instances;
    returns the step."""
    with np.load(path) as z:
        meta = json.loads(bytes(z["meta"]).decode())
        fields = z["fields"]
    own = [[int(i.L), int(i.seed), float(i.a), float(i.a_step)] for i in batch.inst]
    if own != meta["instances"] or meta["precision"] != batch.precision:
        raise ValueError("checkpoint does not match this batch's instances or precision")
    batch.upload(fields, step=int(meta["step"]))
    return int(meta["step"])
