"""Regenerate tests/golden/*.json from the reference's own draw path.

Run in a checkout where the reference tree exists (it is read in place, never
copied): builds oracle/_ref with oracle/Makefile, renders every pinned scene of
tests/scenes_edge.py through the reference ICD in its serial (primitive-order)
mode and records, per target, the SHA-256 of the BGRA8 colour and D32 depth
bytes plus the reference's rasterizer counters.  Scenes whose behaviour has no
reference implementation (trilinear filtering) are recorded from the
project's CPU restatement in spec.json and marked unpinned.

    python tests/golden/make_golden.py [--reference /root/reference]
"""
import argparse
import hashlib
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)
sys.path.insert(0, os.path.dirname(HERE))

from oracle import loader  # noqa: E402
import scenes_edge  # noqa: E402


def digest(cols, deps):
    return [{"color": hashlib.sha256(c.tobytes()).hexdigest(),
             "depth": hashlib.sha256(d.tobytes()).hexdigest()} for c, d in zip(cols, deps)]


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default="/root/reference")
    args = ap.parse_args()
    loader.build_reference(args.reference)
    ref = loader.Reference()
    golden = {}
    for name in scenes_edge.ALL_PINNED:
        h = scenes_edge.build(ref.lib, name)
        cols, deps, counters, _ = ref.render(h, threaded=False)
        golden[name] = {"targets": digest(cols, deps), "counters": counters,
                        "sizes": h.targets()}
        h.close()
        print(name, counters)
    with open(os.path.join(HERE, "golden.json"), "w") as fh:
        json.dump({"source": "reference draw path built from its sources (oracle/_ref), serial mode",
                   "scenes": golden}, fh, indent=1, sort_keys=True)
    orc = loader.Oracle()
    spec = {}
    for name in scenes_edge.SPEC_SCENES:
        h = scenes_edge.build(orc.lib, name)
        cols, deps, counters = orc.render(h)
        spec[name] = {"targets": digest(cols, deps), "counters": counters, "sizes": h.targets()}
        h.close()
        print(name, counters)
    with open(os.path.join(HERE, "spec.json"), "w") as fh:
        json.dump({"source": "project CPU restatement (parity unpinned: no reference implementation)",
                   "scenes": spec}, fh, indent=1, sort_keys=True)


if __name__ == "__main__":
    main()
