"""SVD-event log: one JSON record per two-site factorisation, gzip-compressed
JSON lines.  Drop-in for the reference's event stream (writer
src/atlas_q/tools_qih/svd_logger.py:11-41, record fields emitted at
src/atlas_q/tools_qih/tn_core.py:247-274):

* enabled by the same environment variable, ``QIH_SVD_LOG_DIR`` (or by passing
  a logger to ``AdaptiveMPS.svd_logger``);
* file ``svd_events_<YYYYmmdd_HHMMSS>_<pid>.jsonl.gz`` in that directory;
* every record carries ``host``, ``pid``, ``run_ts`` and the reference's
  fields ``kind="svd_spectrum"``, ``i``, ``j``, ``pre_rank``, ``chi_max``,
  ``tol``, ``adaptive``, ``entangler`` (env ``QIH_ENTANGLER``),
  ``total_weight`` (sum of sigma^2), ``S_top128`` (leading singular values,
  zero-padded to 128) and ``adaptive_keep`` (the kept rank).

Records written by this package add ``step`` (the instance's gate counter),
``chi_left`` / ``chi_right`` and, when the rank predictor's features were
computed for the gate, ``features`` (the predictor's five inputs) and
``full`` (the rank the eigensolver would compute without a prediction):
extra keys a reader of the reference's format ignores.  ``read_events``
reads either producer's files.
"""
import gzip
import json
import os
import threading
import time
from pathlib import Path
from typing import Iterator, List, Optional

TOP = 128


class SVDEventLogger:
    """Appends records to one ``.jsonl.gz`` file (thread-safe, flushed per record)."""

    def __init__(self, out_dir: str):
        self.dir = Path(out_dir)
        self.dir.mkdir(parents=True, exist_ok=True)
        run_ts = time.strftime("%Y%m%d_%H%M%S")
        pid = os.getpid()
        self.path = self.dir / f"svd_events_{run_ts}_{pid}.jsonl.gz"
        self._fh = gzip.open(self.path, "at", encoding="utf-8")
        self._lock = threading.Lock()
        host = os.uname().nodename if hasattr(os, "uname") else "unknown"
        self._meta = {"host": host, "pid": pid, "run_ts": run_ts}

    def log(self, **fields):
        rec = dict(self._meta)
        rec.update(fields)
        line = json.dumps(rec, separators=(",", ":"))
        with self._lock:
            self._fh.write(line + "\n")
            self._fh.flush()

    def spectrum(self, *, bond: int, pre_rank: int, chi_max: int, tol: float, total_weight: float,
                 sigma: List[float], keep: int, step: int, chi_left: int, chi_right: int,
                 features: Optional[List[float]] = None, full: Optional[int] = None):
        top = [float(abs(x)) for x in sigma[:TOP]]
        top += [0.0] * (TOP - len(top))
        extra = {}
        if features is not None:
            extra["features"] = [float(x) for x in features]
            extra["full"] = int(full)
        self.log(kind="svd_spectrum", i=int(bond), j=int(bond) + 1, pre_rank=int(pre_rank), chi_max=int(chi_max),
                 tol=float(tol), adaptive=True, entangler=os.getenv("QIH_ENTANGLER", "unknown"),
                 total_weight=float(total_weight), S_top128=top, adaptive_keep=int(keep), step=int(step),
                 chi_left=int(chi_left), chi_right=int(chi_right), **extra)

    def close(self):
        with self._lock:
            self._fh.close()


def get_logger() -> Optional[SVDEventLogger]:
    """A logger writing to ``$QIH_SVD_LOG_DIR``, or None when it is unset."""
    out = os.getenv("QIH_SVD_LOG_DIR")
    return SVDEventLogger(out) if out else None


def read_events(path_or_dir: str, kind: str = "svd_spectrum") -> Iterator[dict]:
    """Records of one file, or of every ``svd_events_*.jsonl.gz`` in a directory
    (sorted by name), filtered by ``kind``."""
    p = Path(path_or_dir)
    files = sorted(p.glob("svd_events_*.jsonl.gz")) if p.is_dir() else [p]
    for f in files:
        with gzip.open(f, "rt", encoding="utf-8") as fh:
            for line in fh:
                line = line.strip()
                if not line:
                    continue
                rec = json.loads(line)
                if kind is None or rec.get("kind") == kind:
                    yield rec
