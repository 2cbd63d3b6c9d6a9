"""Ensemble batching: plaquettes, Polyakov loop and B^2 of many gauge fields
of uneven volume in one persistent, graph-captured launch (no reference
counterpart: the reference's ``magnetic`` app reads and measures
configurations one at a time, app/magnetic.f90:109-140).

* :class:`Ensemble` -- device task list over a list of
  :class:`~flue_gb300.field.GaugeField` of one precision; ``run()`` replays a
  CUDA graph (memset of the scheduler counters + one cooperative persistent
  kernel + per-field finisher, or in pipeline mode the per-field kernel
  pipelines) and returns per-field observables.
* :func:`autotune` -- the project's tile tuner: times candidate (columns per
  item, block size, blocks per SM) on the actual ensemble and caches the
  winner in a JSON file keyed by GPU name and ensemble signature.
* :func:`shard_by_volume` / :func:`run_sharded` -- split an ensemble across
  ranks (greedy longest-processing-time by volume) and gather the scalars on
  every rank; no data-path collective, only the final gather.
"""
from __future__ import annotations

import ctypes
import hashlib
import json
import os
import time
from typing import Dict, List, Sequence

import numpy as np
import torch

from . import _lib
from .field import GaugeField, _stream_handle

NOBS = 6
CANDIDATES = [(t, b, m) for t in (1, 2, 4, 8, 16) for b in (128, 256) for m in (1, 2, 4)]


def _cache_path() -> str:
    d = os.environ.get("FLUE_CACHE_DIR") or os.path.join(os.path.expanduser("~"), ".cache", "flue_gb300")
    os.makedirs(d, exist_ok=True)
    return os.path.join(d, "ensemble_tiles.json")


def _signature(fields: Sequence[GaugeField], with_b2: bool) -> str:
    dev = torch.cuda.get_device_name(fields[0].device)
    desc = [f"{f.prec}:{'x'.join(map(str, f.dims))}" for f in fields]
    h = hashlib.sha1(("|".join(desc) + f"|b2={int(with_b2)}").encode()).hexdigest()[:16]
    return f"{dev}|{h}"


class Ensemble:
    """``mode="persistent"`` (default): ONE cooperative persistent launch (plus
    a per-field finisher) over all fields: blocks take tasks from a counter --
    the straight lines of a time slab, the line-based 5-loop F and B^2
    partials of a chunk of the slab (waiting, bounded, only on the lines of
    that slab), and plaquettes / Polyakov loops of a run of time columns.
    ``mode="pipeline"``: per field the device entry points (plaquettes,
    Polyakov loop, line-based B^2 on time slabs) with one library workspace
    of the largest field's size, all captured into one graph; same outputs,
    several kernels per field.  Both modes replay from a CUDA graph.  A
    scheduler wait that runs out (which does not happen in a healthy run)
    makes the outputs NaN and ``run`` raise."""

    def __init__(self, fields: Sequence[GaugeField], tile=None, block=128, blocks_per_sm=3, with_b2=True,
                 tune=False, mode="persistent"):
        if not fields:
            raise ValueError("empty ensemble")
        precs = {f.prec for f in fields}
        if len(precs) != 1:
            raise TypeError("all fields of an ensemble must have the same precision")
        self.fields = list(fields)
        self.with_b2 = bool(with_b2)
        self.device = fields[0].device
        if mode not in ("persistent", "pipeline"):
            raise ValueError("mode must be 'persistent' or 'pipeline'")
        self.mode = mode
        if mode == "pipeline":
            tile = 0  # the C ABI's pipeline mode
        elif tune:
            tile, block, blocks_per_sm = autotune(self.fields, with_b2=self.with_b2)
        elif tile is None:
            # measured on GB300, 96 fields of 16^3x32 .. 32^3x64: 16 columns per
            # plaquette / Polyakov task, 128 threads, 3 blocks per SM: 111 ms
            # FP32 (c64) and 3.46 s FP64 per evaluation (pipeline mode 115 ms,
            # 3.48 s); 4 columns 118 ms, 2 blocks per SM 146 ms
            tile = 16
        self.config = (int(tile), int(block), int(blocks_per_sm))
        self._descs = (_lib.FlueField * len(fields))(*[f.descriptor() for f in fields])
        self._h = ctypes.c_void_p()
        with torch.cuda.device(self.device):
            _lib.call("flue_ensemble_create", ctypes.byref(self._h), self._descs, len(fields), *self.config,
                      int(self.with_b2))
        self.out = torch.zeros((len(fields), NOBS), dtype=torch.float64, device=self.device)
        self._captured = False

    @property
    def items(self) -> int:
        return _lib.load().flue_ensemble_items(self._h)

    def capture(self):
        with torch.cuda.device(self.device):
            _lib.call("flue_ensemble_capture", self._h, ctypes.c_void_p(self.out.data_ptr()))
        self._captured = True

    def launch(self, graph=True):
        """Queue one evaluation on the current stream (no synchronisation)."""
        with torch.cuda.device(self.device):
            if graph:
                if not self._captured:
                    self.capture()
                _lib.call("flue_ensemble_replay", self._h, _stream_handle())
            else:
                _lib.call("flue_ensemble_run", self._h, ctypes.c_void_p(self.out.data_ptr()), _stream_handle())

    def run(self, graph=True) -> np.ndarray:
        self.launch(graph)
        raw = self.out.cpu().numpy()
        if np.isnan(raw).any():
            raise _lib.FlueError("flue_ensemble_run", _lib.FLUE_ERR_TIMEOUT,
                                 "a wait of the persistent scheduler ran out; outputs are NaN")
        return raw

    def observables(self, graph=True) -> List[Dict[str, float]]:
        """Per field: mean plaquettes <Re Tr P>/3 (total, spatial, temporal),
        the mean Polyakov loop <Tr P_t>/3 (complex) and B^2."""
        raw = self.run(graph)
        res = []
        for f, r in zip(self.fields, raw):
            V = float(f.volume)
            V3 = V / f.nt
            sp, tp = r[0] / (3 * V), r[1] / (3 * V)
            res.append({"dims": f.dims, "plaq": (sp + tp) / 2 / 3, "splaq": sp / 3, "tplaq": tp / 3,
                        "polyakov": complex(r[2], r[3]) / V3 / 3, "b2": r[4] if self.with_b2 else None,
                        "sum_re_tr_p_spatial": r[0], "sum_re_tr_p_temporal": r[1], "sum_re_tr_polyakov": r[2]})
        return res

    def close(self):
        if self._h:
            _lib.call("flue_ensemble_destroy", self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def autotune(fields: Sequence[GaugeField], with_b2=True, candidates=CANDIDATES, reps=2, use_cache=True):
    """Pick (tile columns, block, blocks per SM) by timing each candidate on
    the ensemble itself; the choice is cached per GPU and ensemble."""
    key = _signature(fields, with_b2)
    path = _cache_path()
    cache = {}
    if use_cache and os.path.exists(path):
        try:
            cache = json.load(open(path))
        except (OSError, ValueError):
            cache = {}
        if key in cache:
            return tuple(cache[key]["config"])
    best, best_ms, table = None, float("inf"), []
    for cand in candidates:
        ens = Ensemble(fields, tile=cand[0], block=cand[1], blocks_per_sm=cand[2], with_b2=with_b2)
        ens.launch(graph=False)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            ens.launch(graph=False)
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / reps
        table.append((cand, ms))
        if ms < best_ms:
            best, best_ms = cand, ms
        ens.close()
    cache[key] = {"config": list(best), "ms": best_ms, "when": time.time(),
                  "table": [[list(c), m] for c, m in table]}
    try:
        json.dump(cache, open(path, "w"), indent=1)
    except OSError:
        pass
    return best


# ---------------------------------------------------------------------------
# multi-rank sharding (independent fields; only the scalars are gathered)
# ---------------------------------------------------------------------------
def shard_by_volume(volumes: Sequence[int], world_size: int) -> List[List[int]]:
    """Greedy longest-processing-time assignment of field indices to ranks,
    balancing the total volume; deterministic (ties broken by index)."""
    order = sorted(range(len(volumes)), key=lambda i: (-volumes[i], i))
    load = [0] * world_size
    shards: List[List[int]] = [[] for _ in range(world_size)]
    for i in order:
        r = min(range(world_size), key=lambda k: (load[k], k))
        shards[r].append(i)
        load[r] += volumes[i]
    return [sorted(s) for s in shards]


def run_sharded(make_field, volumes: Sequence[int], rank: int, world_size: int, compute=None, group=None):
    """Evaluate the fields assigned to this rank and gather every field's row
    of results (index order) on all ranks.  ``make_field(i)`` builds field i
    on this rank's device; ``compute(list_of_fields) -> array (n, NOBS)``
    defaults to an :class:`Ensemble` run.  Uses torch.distributed (any
    backend) only for the final all_gather_object."""
    import torch.distributed as dist

    shards = shard_by_volume(volumes, world_size)
    mine = shards[rank]
    if compute is None:
        def compute(fs):
            return Ensemble(fs).run() if fs else np.zeros((0, NOBS))
    rows = compute([make_field(i) for i in mine]) if mine else np.zeros((0, NOBS))
    local = {i: [float(v) for v in row] for i, row in zip(mine, np.asarray(rows).reshape(len(mine), -1))}
    gathered = [None] * world_size
    if world_size > 1:
        dist.all_gather_object(gathered, local, group=group)
    else:
        gathered = [local]
    merged = {}
    for part in gathered:
        merged.update(part)
    return np.array([merged[i] for i in range(len(volumes))])
