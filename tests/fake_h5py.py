"""An in-memory stand-in for the part of h5py that SynchRad's file paths use.

h5py is installed neither here nor on the GPU host, so the HDF5 code paths
(spectrum output, ``Args`` round trip, track-file input) are exercised
against this module: ``File(name, mode)`` opens a dict of absolute dataset
paths kept in ``FILES``; ``f[path] = value`` stores a numpy copy,
``f[path][()]`` reads it back (``f[path][i, j]`` a slice of it, ``.shape`` its
shape), groups answer ``keys()`` with their children.
String values come back as ``bytes``, as h5py returns variable-length
strings.
"""
from __future__ import annotations

import numpy as np

FILES: dict = {}


def _stored(value):
    if isinstance(value, str):
        return value.encode()
    return np.array(value)


class _Node:
    def __init__(self, store, path):
        self._store, self._path = store, path

    def _children(self):
        pre = self._path + "/" if self._path else ""
        return sorted({k[len(pre):].split("/")[0] for k in self._store if k.startswith(pre)})

    def keys(self):
        if self._path in self._store:
            raise TypeError(f"{self._path} is a dataset")
        return self._children()

    @property
    def shape(self):
        return np.shape(self._store[self._path])

    def __getitem__(self, key):
        if not isinstance(key, str) and key != ():
            return np.array(self._store[self._path][key])   # a slice of a dataset
        if key == ():
            if self._path not in self._store:
                raise KeyError(self._path)
            v = self._store[self._path]
            return v if isinstance(v, bytes) else (v[()] if v.ndim == 0 else v.copy())
        path = f"{self._path}/{key}" if self._path else str(key)
        if path not in self._store and not any(k.startswith(path + "/") for k in self._store):
            raise KeyError(path)
        return _Node(self._store, path)

    def __contains__(self, key):
        path = f"{self._path}/{key}" if self._path else str(key)
        return path in self._store or any(k.startswith(path + "/") for k in self._store)


class File(_Node):
    def __init__(self, name, mode="r"):
        name = str(name)
        if mode == "w":
            FILES[name] = {}
        elif name not in FILES:
            raise FileNotFoundError(name)
        super().__init__(FILES[name], "")

    def __setitem__(self, path, value):
        self._store[str(path).strip("/")] = _stored(value)

    def close(self):
        pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
