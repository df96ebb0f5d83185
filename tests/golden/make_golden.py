"""Generates tests/golden/golden.json: SHA-256 digests (and sizes) of the
oracle's encodes of seeded synthetic pages, plus tests/golden/cfg0.j2k, the
full 512x512 gray q100 codestream.

The oracle is pinned to the reference by tests/test_oracle_kat.py; these
digests freeze its whole-codestream output so that both the oracle (CPU
suite) and the CUDA path (GPU suite) are checked against the same bytes.

    python tests/golden/make_golden.py
"""
import hashlib
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from jp2lam_gb300._native import synth_page  # noqa: E402
from tests import oracle_lib  # noqa: E402

# (name, w, h, ncomp, quality, format, seed, glyphs, photo_w, photo_h)
CASES = [
    ("cfg0_512_gray_q100_j2k", 512, 512, 1, 100, 0, 0, 400, 0, 0),
    ("gray_300x200_q85_jp2", 300, 200, 1, 85, 1, 11, -1, 90, 60),
    ("gray_300x200_q50_j2k", 300, 200, 1, 50, 0, 12, -1, 90, 60),
    ("gray_257x129_q20_j2k", 257, 129, 1, 20, 0, 13, -1, 64, 48),
    ("rgb_200x150_q75_jp2", 200, 150, 3, 75, 1, 14, -1, 80, 60),
    ("rgb_130x97_q100_j2k", 130, 97, 3, 100, 0, 15, -1, 40, 30),
    ("rgb_96x64_q42_j2k", 96, 64, 3, 42, 0, 16, -1, 32, 24),
    ("gray_640x480_q99_j2k", 640, 480, 1, 99, 0, 17, -1, 200, 150),
    ("gray_33x17_q85_j2k", 33, 17, 1, 85, 0, 18, -1, 0, 0),
    ("gray_7x5_q100_j2k", 7, 5, 1, 100, 0, 19, -1, 0, 0),
]


def main():
    orc = oracle_lib.load()
    out = {"generator": "tests/golden/make_golden.py", "cases": []}
    for name, w, h, c, q, fmt, seed, glyphs, pw, ph in CASES:
        px = synth_page(w, h, c, seed, glyphs=glyphs, photo_w=pw, photo_h=ph)
        data = orc.encode(px, w, h, c, q, fmt=fmt, threads=4)
        out["cases"].append({"name": name, "w": w, "h": h, "ncomp": c, "quality": q, "format": fmt,
                             "seed": seed, "glyphs": glyphs, "photo_w": pw, "photo_h": ph,
                             "input_sha256": hashlib.sha256(px.tobytes()).hexdigest(),
                             "sha256": hashlib.sha256(data).hexdigest(), "size": len(data)})
        if name.startswith("cfg0"):
            open(os.path.join(HERE, "cfg0.j2k"), "wb").write(data)
        print(name, len(data))
    with open(os.path.join(HERE, "golden.json"), "w") as f:
        json.dump(out, f, indent=1)
        f.write("\n")


if __name__ == "__main__":
    main()
