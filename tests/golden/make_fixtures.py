"""Generates the golden fixtures of tests/golden/ from the reference checkout.

Run once where the reference is present:  python tests/golden/make_fixtures.py <reference checkout>
(the path is required: the directory holding the reference's test/ and data/). It decodes the reference's pinned results test/*.res (UTF-16LE dumps of the stdout report of an
earlier MaBoSSG build: final points, fixed points, then per window the entropy, the transition
entropy and the state probabilities) into <model>.json, and copies the four input models
data/<model>.bnd/.cfg into models/, so the tests need neither the reference nor its build.
Large reports are thinned: every window is kept for the small models; for Montagud every 10th
window, the 40 most likely fixed points, and the total fixed-point mass.
"""
from __future__ import annotations

import json
import os
import shutil
import sys

MODELS = {
    "cellcycle": "cellcycle",
    "sizek": "sizek",
    "metastasis": "metastasis",
    "Montagud2022_Prostate_Cancer": "montagud",
}


def parse_res(text: str) -> dict:
    lines = [l.strip() for l in text.lstrip("﻿").splitlines() if l.strip()]
    out = {"final": {}, "fixed": {}, "windows": []}
    section = None
    win = None
    for l in lines:
        if l == "final points:":
            section = "final"
            continue
        if l == "fixed points:":
            section = "fixed"
            continue
        if l.startswith("window ("):
            a, b = l[len("window ("):-1].split(",")
            win = {"start": float(a), "end": float(b), "probs": {}}
            out["windows"].append(win)
            section = "window"
            continue
        if l.startswith("entropy:"):
            win["entropy"] = float(l.split(":")[1])
            continue
        if l.startswith("transition entropy:"):
            win["th"] = float(l.split(":")[1])
            continue
        p, state = l.split(" ", 1)
        key = "" if state == "<nil>" else "|".join(state.split("-"))
        if section == "window":
            win["probs"][key] = float(p)
        else:
            out[section][key] = float(p)
    return out


def main(ref: str):
    here = os.path.dirname(os.path.abspath(__file__))
    os.makedirs(os.path.join(here, "models"), exist_ok=True)
    for src, name in MODELS.items():
        with open(os.path.join(ref, "test", src + ".res"), "rb") as f:
            res = parse_res(f.read().decode("utf-16-le"))
        res["fixed_total"] = sum(res["fixed"].values())
        res["fixed_count"] = len(res["fixed"])
        if name == "montagud":
            res["windows"] = [w for i, w in enumerate(res["windows"]) if i % 10 == 9]
            top = sorted(res["fixed"].items(), key=lambda kv: -kv[1])[:40]
            res["fixed"] = dict(top)
        res["model"] = name
        with open(os.path.join(here, name + ".json"), "w") as f:
            json.dump(res, f, separators=(",", ":"), sort_keys=True)
        for ext in ("bnd", "cfg"):
            shutil.copyfile(os.path.join(ref, "data", f"{src}.{ext}"), os.path.join(here, "models", f"{name}.{ext}"))
        print(name, len(res["windows"]), "windows", len(res["fixed"]), "fixed points")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_fixtures.py <reference checkout (holds test/ and data/)>")
    main(sys.argv[1])
