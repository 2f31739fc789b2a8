"""Loads the committed golden fixtures (tests/golden/), made by tests/golden/make_golden.py
from the reference library compiled unmodified."""
import json
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def known_answers():
    with open(os.path.join(GOLDEN, "known_answers.json")) as f:
        cases = json.load(f)
    out = []
    for c in cases:
        d = dict(c)
        d["indices"] = np.array(c["indices"], np.uint32)
        d["positions"] = np.array(c["positions"], np.float32)
        for k, dt in (("attributes", np.float32), ("weights", np.float32), ("lock", np.uint8), ("expect", np.uint32)):
            d[k] = None if c[k] is None else np.array(c[k], dt)
        d["ref_output"] = np.array(c["ref_output"], np.uint32)
        out.append(d)
    return out


def seeded_cases():
    z = np.load(os.path.join(GOLDEN, "seeded_cases.npz"))
    meta = json.loads(str(z["meta"]))
    out = []
    for i, m in enumerate(meta):
        d = dict(m)
        for k in ("indices", "positions", "attributes", "weights", "expect"):
            key = f"{i}_{k}"
            d[k] = z[key] if key in z else None
        out.append(d)
    return out


def compaction_cases():
    z = np.load(os.path.join(GOLDEN, "compaction_cases.npz"))
    out = []
    for i in range(int(z["count"])):
        prefix = f"{i}_"
        d = {k[len(prefix):]: z[k] for k in z.files if k.startswith(prefix)}
        d["kind"] = str(d["kind"])
        out.append(d)
    return out


def clod_cases():
    z = np.load(os.path.join(GOLDEN, "clod_cases.npz"))
    out = []
    for i in range(int(z["count"])):
        prefix = f"{i}_"
        out.append({k[len(prefix):]: z[k] for k in z.files if k.startswith(prefix)})
    return out


def update_cases():
    z = np.load(os.path.join(GOLDEN, "update_cases.npz"))
    out = []
    for i in range(int(z["count"])):
        prefix = f"{i}_"
        d = {k[len(prefix):]: z[k] for k in z.files if k.startswith(prefix)}
        d["name"] = str(d["name"])
        d["kind"] = str(d["kind"])
        out.append(d)
    return out


def meshlet_cases():
    """meshopt_buildMeshletsFlex golden cases: each with its mesh's indices and positions."""
    z = np.load(os.path.join(GOLDEN, "meshlet_cases.npz"))
    out = []
    for i in range(int(z["count"])):
        prefix = f"{i}_"
        d = {k[len(prefix):]: z[k] for k in z.files if k.startswith(prefix)}
        d["name"] = str(d["name"])
        j = int(d["mesh"])
        d["indices"] = z[f"mesh{j}_indices"]
        d["positions"] = z[f"mesh{j}_positions"]
        out.append(d)
    return out
