"""Loader for the golden vectors in tests/golden/*.npz (see make_golden.py)."""
from __future__ import annotations

import json
from dataclasses import dataclass
from pathlib import Path

import numpy as np

GOLDEN = Path(__file__).resolve().parent / "golden"
KEYS = ("x", "y", "z", "ux", "uy", "uz")


@dataclass
class GoldenCase:
    name: str
    args: dict
    call: dict
    tracks: list
    expected: dict
    total_weight: float
    snap_iterations: np.ndarray
    omega: np.ndarray | None = None   # the axis the expected values were computed on

    def fresh_tracks(self):
        """Deep copies in the reference list format (the call may mutate weights)."""
        out = []
        for t in self.tracks:
            tt = [a.copy() for a in t[:6]] + list(t[6:])
            out.append(tt)
        return out

    def fresh_args(self):
        a = json.loads(json.dumps(self.args))
        g = a["grid"]
        a["grid"] = [tuple(v) for v in g]
        return a


def names():
    """The spectrum cases (the *_golden.npz files hold the host-logic and
    converter vectors)."""
    return sorted(p.stem for p in GOLDEN.glob("*.npz") if not p.stem.endswith("_golden"))


def load(name: str) -> GoldenCase:
    d = np.load(GOLDEN / f"{name}.npz")
    meta = json.loads(str(d["meta_json"]))
    tracks = []
    for i in range(meta["n_tracks"]):
        arrs = [d[f"track{i}_{k}"] for k in KEYS]
        w, its = d[f"track{i}_meta"]
        t = arrs + [float(w)]
        if its >= 0:
            t.append(int(its))
        tracks.append(t)
    call = dict(meta["call"])
    if call.get("it_range") is not None:
        call["it_range"] = tuple(call["it_range"])
    expected = {k[4:]: d[k] for k in d.files if k.startswith("out_")}
    return GoldenCase(name, meta["args"], call, tracks, expected,
                      float(d["total_weight"]), d["snap_iterations"],
                      d["omega"] if "omega" in d.files else None)
