"""Writes tests/golden/ic_examples.json from the reference itself.

Runs the reference's DataManager (compiled from its sources into
oracle/_ref/libag2ref.so by oracle/Makefile) on
  * the four example initial conditions shipped with the reference
    (input_data/Example), read with loadICs: per-field sha256 of the loaded
    particles (makeGal, which the reader shuffles, in canonical order);
  * oracle.snapio.random_particles(1000, seed=3), written with saveData in
    each snapshot format for count 1000 and 777: sha256 of the file bytes
    (the ag/agc/age header's 4 uninitialised padding bytes zeroed).
Usage: python tests/golden/make_ic_golden.py [reference checkout]  (default: $AG2_REF, else the
location oracle/Makefile names)
"""
import hashlib
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", "..", "oracle"))
import oracle  # noqa: E402
import snapio as S  # noqa: E402

EXAMPLES = [("gassphere_littleendian.dat", "gadget"), ("galaxy_littleendian.dat", "gadget"),
            ("galiC_M1_22k.dat", "gadget"), ("galaxy_gas.dat", "makeGal")]


def main():
    ref = sys.argv[1] if len(sys.argv) > 1 else oracle.reference_checkout()
    assert ref, "no reference checkout: set AG2_REF or pass its path"
    assert S.ref_lib() is not None, "build oracle/_ref first (make -C oracle ref)"
    out = {"examples": {}, "snapshots": {}}
    for name, fmt in EXAMPLES:
        path = os.path.join(ref, "input_data", "Example", name)
        p, ok = S.ref_load(path, fmt, 1 << 20)
        order = S.canonical_order(p) if fmt == "makeGal" else None
        out["examples"][name] = {"format": fmt, "n": int(len(p["mass"])), "reader_ok": ok,
                                 "sha256": S.field_digest(p, order)}
    p = S.random_particles(1000, 3)
    for fmt in ("ag", "agc", "age", "gadget"):
        for count in (1000, 777):
            b = bytearray(S.ref_save(fmt, p, count, 1.5, 2.5, 3.5))
            if fmt != "gadget":
                b[12:16] = bytes(4)
            out["snapshots"][f"{fmt}_{count}"] = {"bytes": len(b), "sha256": hashlib.sha256(b).hexdigest()}
    with open(os.path.join(HERE, "ic_examples.json"), "w") as f:
        json.dump(out, f, indent=1, sort_keys=True)
        f.write("\n")


if __name__ == "__main__":
    main()
