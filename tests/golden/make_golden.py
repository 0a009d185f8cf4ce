"""Regenerate the golden vectors in this directory from the reference itself.

Builds the pin harnesses of oracle/ref_pin (``make -C oracle ref``), which compile the
reference sources where they lie and run the reference's own FP64 CPU code, then
gzips their output here. Needs the reference checkout: REF_DIR on the command line, else
$FPDE_REFERENCE_DIR, else a directory named "reference" beside the repository; the fixtures
themselves are committed so tests never need it.

    python tests/golden/make_golden.py [REF_DIR] [--only gamma|richards|richards_ct|spacefrac|spacefrac3d|lod_vartau|kat|kat_alg2|frdo_kat]

The richards, richards_ct, spacefrac, spacefrac3d, lod_vartau, kat (the column and the 3D known
answers) and kat_alg2 (the 3D known answer with the series history) scenarios, and frdo_kat
(fr_do's runs at its defaults), run only with --only (each sets its own solver mode). The
harness's kat40 scenario (the 40 x 40 x 40 known answer, 8 MB) is written by its test into a
temporary folder instead.

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
    args = [a for a in sys.argv[1:] if not a.startswith("--")]
    only = sys.argv[sys.argv.index("--only") + 1] if "--only" in sys.argv else None
    if only:
        args = [a for a in args if a != only]
    sys.path.insert(0, ROOT)
    import __graft_entry__
    ref_dir = args[0] if args else __graft_entry__.reference_dir()
    if not ref_dir:
        raise SystemExit("no reference checkout: pass REF_DIR or set FPDE_REFERENCE_DIR")
    subprocess.check_call(["make", "-C", os.path.join(ROOT, "oracle"), "ref",
                           f"REF_DIR={ref_dir}"])
    tmp = tempfile.mkdtemp(prefix="fpde_golden_")
    try:
        if only == "frdo_kat":   # fr_do's default runs (pin_frdo kat)
            subprocess.check_call([os.path.join(ROOT, "oracle", "_ref", "pin_frdo"), "kat", tmp], cwd=tmp)
        elif only:               # one scenario of the fpde harness (e.g. gamma)
            subprocess.check_call([os.path.join(ROOT, "oracle", "_ref", "pin_fpde"), only, tmp], cwd=tmp)
        for exe in (() if only else ("pin_fpde", "pin_frdo")):
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
