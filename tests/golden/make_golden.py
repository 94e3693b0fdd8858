"""Generate the golden vectors in tests/golden/ from the reference itself.

Runs the reference's own C code (compiled in place from the reference tree by
`make -C oracle ref` into oracle/_ref/libmtgpref.so) and stores what it
produces, so that the CPU restatement (oracle/) can be pinned on machines
where the reference tree is absent.  The sequences mirror the reference's
own known-answer program (mtgp32-fast.c:436-514, mtgp64-fast.c:430-508):
init(seed=1), init_by_array({1,2,3,4}), init_by_str("\\1\\2\\3\\4") followed
by every float kind; plus a key with bytes >= 0x80, and a jump by the shipped
JUMP3_162 polynomial (mtgp32-fast-jump.c:51-79).

    make -C oracle ref && python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "..", ".."))
from mtgp_gb300.params import load_table, jump_string  # noqa: E402
from oracle.bind import Reference  # noqa: E402

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "ref_vectors.npz")

CASES = [  # (table, index, outputs per sequence)
    ("mtgp32_fast_11213", 0, 1000), ("mtgp32_fast_11213", 127, 256),
    ("mtgp32_fast_23209", 0, 256), ("mtgp32_fast_44497", 0, 256),
    ("mtgp32dc_fast_11213", 0, 256),
    ("mtgp64dc_fast_11213", 0, 1000), ("mtgp64dc_fast_11213", 199, 256),
    ("mtgp64dc_cuda_fast_11213", 0, 256), ("mtgp64_fast_23209", 0, 256),
    ("mtgp64_fast_44497", 0, 256), ("mtgp64_fast_110503", 0, 256),
]
HIGH_KEY = b"\x80\xff\x7fMTGP\xc3\xa9"


def main():
    ref = Reference()
    out = {}
    for table, idx, n in CASES:
        p = load_table(table)[idx]
        key = "%s_%d" % (table, idx)
        out[key + "_seed1_uint"] = ref.gen(p, seed=1).fill(0, n)
        out[key + "_array1234_uint"] = ref.gen(p, array=[1, 2, 3, 4]).fill(0, n)
        g = ref.gen(p, string=b"\x01\x02\x03\x04")
        out[key + "_str1234_uint"] = g.fill(0, n)
        for kind in (1, 2, 3, 4):
            out[key + "_str1234_kind%d" % kind] = g.fill(kind, n)
        out[key + "_highkey_uint"] = ref.gen(p, string=HIGH_KEY).fill(0, n)
    for bits, table in ((32, "mtgp32_fast_11213"), (64, "mtgp64dc_fast_11213")):
        p = load_table(table)[0]
        g = ref.gen(p, seed=1234)
        g.fill(0, 777)
        g.fast_jump(jump_string(bits))
        idx, ring = g.ring()
        out["jump%d_idx" % bits] = np.array([idx])
        out["jump%d_ring" % bits] = ring
        out["jump%d_next_uint" % bits] = g.fill(0, 512)
    np.savez(OUT, **out)
    print("wrote", OUT, os.path.getsize(OUT), "bytes")


if __name__ == "__main__":
    main()
