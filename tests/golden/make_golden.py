"""Regenerate tests/golden/reference_kat.json from the reference's own code.

Builds oracle/_ref/ref_kat from the reference's host sources (rxnparam,
smolreact, stats, SFMT, dcmt, reaction_cpu) where they lie and stores its
output.  Needs the reference tree ($REF_DIR, else a ``reference`` directory
beside the repository); the committed JSON lets every other machine run the
pins without it.
"""
import json
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", ".."))

from oracle import build as obuild  # noqa: E402


def main():
    exe = obuild.build_ref(force=True)
    if exe is None:
        raise SystemExit("reference tree not found; set REF_DIR")
    tmp = os.path.join(HERE, "..", "..", "oracle", "_ref", "kat.json")
    subprocess.run([exe, tmp], capture_output=True, text=True, check=True)
    with open(tmp) as f:
        data = json.load(f)
    with open(os.path.join(HERE, "reference_kat.json"), "w") as f:
        json.dump(data, f, separators=(",", ":"))
    print("wrote reference_kat.json:", {k: (len(v) if hasattr(v, "__len__") else v) for k, v in data.items()})


if __name__ == "__main__":
    main()
