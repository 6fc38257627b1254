"""On-disk caches of the J-VIE path: assembled operators and matvec schedules.

The reference reuses fN only within a session, keyed by frequency in the body
struct (`RHBM.fN` / `RHBM.freqfN`, fVIE_Assembly.m:109-131, filled by
MARIE_SolveScat.m:825-839).  `OperatorCache` keeps assembled operators on disk
instead, keyed by what determines them: the operator ('N' or 'K'), the grid
(L, M, N), the voxel edge dx, the frequency and the singular-integral
method.  Each entry is a `.npy` file of the FP64 2L x 2M x 2N x q array in
MATLAB's column-major order, beside a `.json` file holding its key; a load
checks that key and the array's shape, so a hash collision or a truncated file
reads as a miss.  Writes go to a temporary file renamed into place, so a
reader never sees a partial entry.

`ScheduleCache` keeps the matvec schedule `Operator.autotune` picks, keyed by
the device name and the FFT grid (the timing depends on nothing else), in one
JSON file, so a deployment tunes each grid once per GPU model.
"""
from __future__ import annotations

import hashlib
import json
import os
import tempfile
from typing import Optional

import numpy as np


def _canonical(key: dict) -> str:
    return json.dumps(key, sort_keys=True)


def operator_key(L: int, M: int, N: int, dx: float, freq: float, op: str = "N", singular: str = "DIRECTFN") -> dict:
    """The values that determine getOPERATORS(r, f, op) on an L x M x N grid of
    edge dx (floats kept exactly, as hexadecimal)."""
    if op not in ("N", "K"):
        raise ValueError("op must be 'N' or 'K'")
    # "scheme" names what 'DIRECTFN' computes (DIRECTFN at Np_1D = 20); entries
    # written before the library computed it (a converged quadrature under the
    # same name) carry no scheme and miss
    return {"op": op, "grid": [int(L), int(M), int(N)], "dx": float(dx).hex(), "freq": float(freq).hex(),
            "singular": singular if op == "N" else None, "scheme": 2}


def _atomic_write(path: str, write) -> None:
    d = os.path.dirname(path) or "."
    fd, tmp = tempfile.mkstemp(dir=d, prefix=".tmp-", suffix=os.path.splitext(path)[1])
    try:
        with os.fdopen(fd, "wb") as fh:
            write(fh)
        os.replace(tmp, path)
    except BaseException:
        if os.path.exists(tmp):
            os.unlink(tmp)
        raise


class OperatorCache:
    """Assembled operators on disk under `directory` (created if absent)."""

    def __init__(self, directory: str):
        self.directory = directory
        os.makedirs(directory, exist_ok=True)

    def _paths(self, key: dict):
        h = hashlib.sha256(_canonical(key).encode()).hexdigest()[:24]
        L, M, N = key["grid"]
        stem = os.path.join(self.directory, "f%s_%dx%dx%d_%s" % (key["op"], L, M, N, h))
        return stem + ".npy", stem + ".json"

    def load(self, key: dict) -> Optional[np.ndarray]:
        """The cached array for key, or None (absent, other key, wrong shape
        or unreadable)."""
        arr_path, key_path = self._paths(key)
        try:
            with open(key_path) as fh:
                if json.load(fh) != json.loads(_canonical(key)):
                    return None
            arr = np.load(arr_path, allow_pickle=False)
        except (OSError, ValueError):
            return None
        L, M, N = key["grid"]
        q = 6 if key["op"] == "N" else 3
        if arr.shape != (2 * L, 2 * M, 2 * N, q) or arr.dtype != np.complex128:
            return None
        return arr

    def store(self, key: dict, arr: np.ndarray) -> None:
        """Writes arr (2L x 2M x 2N x q complex) as the entry of key."""
        L, M, N = key["grid"]
        q = 6 if key["op"] == "N" else 3
        if arr.shape != (2 * L, 2 * M, 2 * N, q):
            raise ValueError("operator shape %s does not match the key's grid" % (arr.shape,))
        arr_path, key_path = self._paths(key)
        data = np.asfortranarray(np.asarray(arr, dtype=np.complex128))
        _atomic_write(arr_path, lambda fh: np.save(fh, data, allow_pickle=False))
        _atomic_write(key_path, lambda fh: fh.write(_canonical(key).encode()))

    def getOPERATORS(self, r, f, op: str = "N", singular: str = "DIRECTFN"):
        """getOPERATORS(r, f, op) (type 'FFTofC') through the cache: a hit is
        read from disk, a miss assembled on the device and stored."""
        from .vie import getOPERATORS

        r = np.asarray(r, dtype=np.float64)
        L, M, N = r.shape[:3]
        dx = float(r[1, 0, 0, 0] - r[0, 0, 0, 0])
        key = operator_key(L, M, N, dx, f, op, singular)
        arr = self.load(key)
        if arr is None:
            arr = getOPERATORS(r, f, op, "FFTofC", singular)
            self.store(key, arr)
        return arr

    def operator(self, L: int, M: int, N: int, dx: float, freq: float, precision: str = "fp64",
                 singular: str = "DIRECTFN", nrhs_max: int = 1):
        """An Operator holding fN for this grid: uploaded from the cache on a
        hit, assembled on the device (and copied to the cache) on a miss."""
        from .vie import Operator

        key = operator_key(L, M, N, dx, freq, "N", singular)
        arr = self.load(key)
        if arr is not None:
            opr = Operator.from_array(arr, precision=precision, nrhs_max=nrhs_max)
            opr.dx, opr.freq = dx, freq
            return opr
        opr = Operator.assemble(L, M, N, dx, freq, precision=precision, singular=singular, nrhs_max=nrhs_max)
        self.store(key, opr.to_array())
        return opr


def device_name() -> str:
    """The CUDA device's name (the schedule cache's key), or 'cuda'."""
    try:
        import torch

        if torch.cuda.is_available():
            return torch.cuda.get_device_name(torch.cuda.current_device())
    except Exception:
        pass
    return "cuda"


class ScheduleCache:
    """Matvec schedules (fuse, fvar, zvar) by device and FFT grid in one JSON
    file."""

    def __init__(self, path: str):
        self.path = path

    @staticmethod
    def key(device: str, L: int, M: int, N: int) -> str:
        return "%s|%dx%dx%d" % (device, 2 * L, 2 * M, 2 * N)

    def _read(self) -> dict:
        try:
            with open(self.path) as fh:
                data = json.load(fh)
            return data if isinstance(data, dict) else {}
        except (OSError, ValueError):
            return {}

    def get(self, key: str):
        v = self._read().get(key)
        if isinstance(v, list) and len(v) == 3 and all(isinstance(i, int) for i in v):
            return tuple(v)
        return None

    def put(self, key: str, schedule) -> None:
        data = self._read()
        data[key] = [int(i) for i in schedule]
        d = os.path.dirname(self.path)
        if d:
            os.makedirs(d, exist_ok=True)
        _atomic_write(self.path, lambda fh: fh.write(json.dumps(data, sort_keys=True, indent=1).encode()))

    def apply(self, opr, device: Optional[str] = None):
        """Pins the cached schedule of opr's grid, or autotunes opr and caches
        the choice.  Returns (schedule, tuned); (None, False) for a plan
        without the FP32 operator, which has nothing to tune."""
        k = self.key(device or device_name(), opr.L, opr.M, opr.N)
        s = self.get(k)
        if s is not None:
            opr.set_schedule(*s)
            return s, False
        s, cands = opr.autotune()
        if not cands:
            return None, False
        self.put(k, s)
        return s, True
