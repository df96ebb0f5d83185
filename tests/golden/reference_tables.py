"""Extract the reference's literal context/probability tables and compare them
with the oracle's tables (which are generated from the standard's rules).

Run in a container where the reference tree is mounted; it writes
``reference_tables.json`` holding SHA-256 digests of each table so that the
tests can check the oracle's (and the CUDA path's) tables without the
reference present.

    python tests/golden/reference_tables.py <path of the jp2lam source tree>
"""
import hashlib
import json
import pathlib
import re
import sys

HERE = pathlib.Path(__file__).resolve().parent


def _ints(text):
    return [int(t, 0) for t in re.findall(r"0x[0-9a-fA-F]+|\d+", text)]


def parse_luts(src):
    zc = src.split("LUT_CTXNO_ZC: [[u8; 512]; 4] = [")[1].split("\n];")[0]
    zc_vals = _ints(zc)
    sc = src.split("LUT_CTXNO_SC: [u8; 256] = [")[1].split("];")[0]
    spb = src.split("LUT_SPB: [u8; 256] = [")[1].split("];")[0]
    return zc_vals, _ints(sc), _ints(spb)


def parse_mq(src):
    body = src.split("MQ_STATES: [MqState; 94] = [")[1].split("];")[0]
    rows = re.findall(r"qeval:\s*(0x[0-9a-fA-F]+),\s*mps:\s*(\d+),\s*nmps:\s*(\d+),\s*nlps:\s*(\d+)", body)
    out = []
    for r in rows:
        out.extend(int(v, 0) for v in r)
    return out


def parse_norms97(src):
    body = src.split("DWT_NORMS_97: [[f64; 10]; 4] = [")[1].split("\n];")[0]
    return [float(v) for v in re.findall(r"\d+\.\d+", body)]


def digest(values, fmt="int"):
    if fmt == "int":
        data = ",".join(str(int(v)) for v in values)
    else:
        data = ",".join(repr(float(v)) for v in values)
    return hashlib.sha256(data.encode()).hexdigest()


def main(ref_root):
    ref = pathlib.Path(ref_root)
    zc, sc, spb = parse_luts((ref / "src/tier1/luts.rs").read_text())
    mq = parse_mq((ref / "src/mq/mod.rs").read_text())
    norms = parse_norms97((ref / "src/dwt/norms.rs").read_text())
    assert len(zc) == 2048, len(zc)
    assert len(sc) == 256 and len(spb) == 256
    assert len(mq) == 94 * 4, len(mq)
    assert len(norms) == 40, len(norms)
    out = {
        "source": "reference src/tier1/luts.rs, src/mq/mod.rs, src/dwt/norms.rs",
        "zc_sha256": digest(zc),
        "sc_sha256": digest(sc),
        "spb_sha256": digest(spb),
        "mq_states_sha256": digest(mq),
        "norms97_sha256": digest(norms, "float"),
    }
    (HERE / "reference_tables.json").write_text(json.dumps(out, indent=1) + "\n")
    print(json.dumps(out, indent=1))


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: reference_tables.py <path of the jp2lam source tree>")
    main(sys.argv[1])
