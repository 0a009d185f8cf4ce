"""Regenerate the golden vectors in this directory from the reference itself.

Builds the pin harnesses of oracle/ref_pin (``make -C oracle ref``), which compile the
reference sources where they lie and run the reference's own FP64 CPU code, then
gzips their output here. Needs the reference checkout (REF_DIR, default the read-only
mount used when these fixtures were made); the fixtures themselves are committed so
tests never need it.

    python tests/golden/make_golden.py [REF_DIR]

The 40-digit weights fixture (fpde_weights_g_exact.fgv.gz) is computed from the time grids of
the fpde_weights_fk* fixtures written here: rerun make_weights_exact.py after this script.
"""
import gzip
import os
import shutil
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))


def main():
    ref_dir = sys.argv[1] if len(sys.argv) > 1 else "/root/reference"
    subprocess.check_call(["make", "-C", os.path.join(ROOT, "oracle"), "ref",
                           f"REF_DIR={ref_dir}"])
    tmp = tempfile.mkdtemp(prefix="fpde_golden_")
    try:
        for exe in ("pin_fpde", "pin_frdo"):
            # fr_do's eq_ex 1 caches series values in ./s_n_t.txt: run inside tmp.
            subprocess.check_call([os.path.join(ROOT, "oracle", "_ref", exe), tmp], cwd=tmp)
        for name in sorted(os.listdir(tmp)):
            if not name.endswith(".fgv"):
                continue
            with open(os.path.join(tmp, name), "rb") as src, \
                    gzip.GzipFile(os.path.join(HERE, name + ".gz"), "wb", 9, mtime=0) as dst:
                shutil.copyfileobj(src, dst)
            print("wrote", name + ".gz")
    finally:
        shutil.rmtree(tmp)


if __name__ == "__main__":
    main()
