"""Autotuner cache: tile shapes chosen by fm_plan_autotune, kept on disk.

The key of an entry is the plan's lowered launch list (fm_plan_describe of
both directions), its compute type, the column count and the device name, so
a cached choice is replayed only for the same launches on the same GPU.
The file lives at $FASTMAT_GB300_CACHE or ~/.cache/fastmat_gb300/tiles.json.
"""

import hashlib
import json
import os
import threading

from . import _native

_lock = threading.Lock()
_mem = {}   # key -> entry, the choices this process has applied already


def cache_path():
    return os.environ.get('FASTMAT_GB300_CACHE') or os.path.join(
        os.path.expanduser('~'), '.cache', 'fastmat_gb300', 'tiles.json')


def _device_name():
    import torch
    return torch.cuda.get_device_name(torch.cuda.current_device())


def _key(plan, num_cols):
    h = hashlib.sha1()
    for d in (_native.FORWARD, _native.BACKWARD):
        h.update(plan.describe(d).encode())
    h.update(('|%d|%d|%s|%d' % (plan.compute_type, num_cols,
                                _device_name(),
                                _native.load().fm_version())).encode())
    return h.hexdigest()


def _load():
    try:
        with open(cache_path()) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _store(db):
    path = cache_path()
    try:
        os.makedirs(os.path.dirname(path), exist_ok=True)
        tmp = path + '.tmp%d' % os.getpid()
        with open(tmp, 'w') as f:
            json.dump(db, f)
        os.replace(tmp, path)
    except OSError:
        pass


def autotune(plan, num_cols, cache=True):
    """Tune (or replay) the tile shapes of both directions of a plan."""
    import torch
    key = _key(plan, num_cols)
    with _lock:
        if cache and key in _mem:
            if getattr(plan, '_tuned_key', None) != key:
                for d in (_native.FORWARD, _native.BACKWARD):
                    plan.set_tiles(d, _mem[key][str(d)])
                plan._tuned_key = key
            return _mem[key]
        db = _load() if cache else {}
        entry = db.get(key)
        if entry is not None:
            try:
                for d in (_native.FORWARD, _native.BACKWARD):
                    plan.set_tiles(d, entry[str(d)])
                _mem[key] = entry
                plan._tuned_key = key
                return entry
            except (ValueError, KeyError):
                pass
        stream = torch.cuda.current_stream().cuda_stream
        entry = {}
        for d in (_native.FORWARD, _native.BACKWARD):
            plan.autotune(d, num_cols, stream)
            entry[str(d)] = plan.tiles(d)
        if cache:
            db = _load()
            db[key] = entry
            _store(db)
            _mem[key] = entry
            plan._tuned_key = key
        return entry
