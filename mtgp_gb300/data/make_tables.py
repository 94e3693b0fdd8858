"""Regenerate the parameter and jump tables shipped in this directory.

The tables are data of the MTGP reference (MersenneTwister-Lab/MTGP v1.1.2):
a generator is defined by its parameter set, so bit-identical output needs
the same numbers.  This script compiles a small dumper against the
reference's own table sources (read in place, never copied) and writes each
table as raw little-endian structs with the reference's layout
(mtgp32-fast.h:47-58, mtgp64-fast.h:46-57), plus the jump polynomials.

    python mtgp_gb300/data/make_tables.py [/path/to/reference]

Only needed when the tables change; the .bin / .txt outputs are committed.
"""
import os
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))

DUMPER = r'''
#include <stdio.h>
#include <string.h>
#include "mtgp32-fast.h"
#include "mtgp64-fast.h"
#include "mtgp32-jump-string.h"
#include "mtgp64-jump-string.h"
#define MTGP32_CHAR11213_H
#include "cuda-sample/mtgp32-char11213.h"
extern mtgp32_params_fast_t mtgp32dc_params_fast_11213[];
extern mtgp64_params_fast_t mtgp64dc_params_fast_11213[];
extern mtgp64_params_fast_t mtgp64dc_cuda_params_fast_11213[];
extern const uint32_t mtgp32_jump_table[];
extern const uint32_t mtgp64_jump_table[];
static void put(const char *dir, const char *name, const void *p, size_t n) {
    char path[4096];
    snprintf(path, sizeof path, "%s/%s", dir, name);
    FILE *f = fopen(path, "wb");
    fwrite(p, 1, n, f);
    fclose(f);
}
int main(int argc, char **argv) {
    const char *d = argv[1];
    put(d, "mtgp32_fast_11213.bin", mtgp32_params_fast_11213, 128 * sizeof(mtgp32_params_fast_t));
    put(d, "mtgp32_fast_23209.bin", mtgp32_params_fast_23209, 128 * sizeof(mtgp32_params_fast_t));
    put(d, "mtgp32_fast_44497.bin", mtgp32_params_fast_44497, 128 * sizeof(mtgp32_params_fast_t));
    put(d, "mtgp32dc_fast_11213.bin", mtgp32dc_params_fast_11213, 200 * sizeof(mtgp32_params_fast_t));
    put(d, "mtgp64_fast_23209.bin", mtgp64_params_fast_23209, 128 * sizeof(mtgp64_params_fast_t));
    put(d, "mtgp64_fast_44497.bin", mtgp64_params_fast_44497, 128 * sizeof(mtgp64_params_fast_t));
    put(d, "mtgp64_fast_110503.bin", mtgp64_params_fast_110503, 128 * sizeof(mtgp64_params_fast_t));
    put(d, "mtgp64dc_fast_11213.bin", mtgp64dc_params_fast_11213, 200 * sizeof(mtgp64_params_fast_t));
    put(d, "mtgp64dc_cuda_fast_11213.bin", mtgp64dc_cuda_params_fast_11213, 200 * sizeof(mtgp64_params_fast_t));
    put(d, "mtgp32_jump_11213.bin", mtgp32_jump_table, 6 * 351 * 4);
    put(d, "mtgp64_jump_11213.bin", mtgp64_jump_table, 6 * 351 * 4);
    put(d, "mtgp32_jump3_162.txt", mtgp32_jump_string, strlen(mtgp32_jump_string));
    put(d, "mtgp64_jump3_162.txt", mtgp64_jump_string, strlen(mtgp64_jump_string));
    put(d, "mtgp32_char_11213.txt", CHAR32_11213, strlen(CHAR32_11213));
    return 0;
}
'''


def main(ref):
    inc = ["-I" + ref, "-I" + os.path.join(ref, "openCL-sample")]
    with tempfile.TemporaryDirectory() as tmp:
        src = os.path.join(tmp, "dump.c")
        with open(src, "w") as f:
            f.write(DUMPER)
        objs = []

        def cc(path, extra, cxx=False):
            obj = os.path.join(tmp, "o%d.o" % len(objs))
            cmd = ["g++" if cxx else "gcc", "-O1", "-w", "-c", path, "-o", obj]
            subprocess.check_call(cmd + inc + extra)
            objs.append(obj)

        cc(src, ["-std=gnu99"])
        cc(os.path.join(ref, "mtgp32-param-fast.c"), ["-std=gnu99"])
        cc(os.path.join(ref, "mtgp64-param-fast.c"), ["-std=gnu99"])
        cc(os.path.join(ref, "cuda-sample/mtgp32dc-param-11213.c"),
           ["-std=gnu99", "-Dmtgpdc_params_11213_num=n1"])
        cc(os.path.join(ref, "openCL-sample/mtgp64dc-param-11213.c"),
           ["-std=gnu99", "-Dmtgpdc_params_11213_num=n2"])
        cc(os.path.join(ref, "cuda-sample/mtgp64dc-param-11213.c"),
           ["-std=gnu99", "-Dmtgpdc_params_11213_num=n3",
            "-Dmtgp64dc_params_fast_11213=mtgp64dc_cuda_params_fast_11213"])
        cc(os.path.join(ref, "openCL-sample/mtgp32-jump-table.cpp"), [], True)
        cc(os.path.join(ref, "openCL-sample/mtgp64-jump-table.cpp"), [], True)
        exe = os.path.join(tmp, "dump")
        subprocess.check_call(["g++", "-o", exe] + objs)
        subprocess.check_call([exe, HERE])
    # 64-bit characteristic polynomial: second line of the shipped text file
    with open(os.path.join(ref, "openCL-sample/characteristic.64.11213.txt")) as f:
        lines = f.read().split("\n")
    with open(os.path.join(HERE, "mtgp64_char_11213.txt"), "w") as f:
        f.write(lines[1].strip())


if __name__ == "__main__":
    # the reference checkout: argument, MTGP_REFERENCE_DIR, or a directory
    # named "reference" beside this repository
    default = os.environ.get("MTGP_REFERENCE_DIR", os.path.normpath(
        os.path.join(HERE, "..", "..", "..", "reference")))
    main(sys.argv[1] if len(sys.argv) > 1 else default)
