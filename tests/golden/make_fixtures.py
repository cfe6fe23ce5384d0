"""Builds the golden fixtures of tests/golden/ from the reference checkout.

Run once in a container that has the reference mounted:
    python tests/golden/make_fixtures.py /path/to/Thesis-EMX-BACH

Copies the reference's only present end-to-end test case (test 1 of
tools/run_test.py:13: science res/test0.fits, template res/test1.fits and
the HOTPANTS goldens tests/test01_conv.fits / tests/test01_sub.fits) and
extracts the test01 global normal matrix printed in tools/cond_num.py:3-298
(293x293, six significant figures) into test01_ksc_matrix.npy.  The
reference is MIT licensed (MindRoad Ost AB 2024; Lells & Wang 2023); the data
files are reproduced unchanged.
"""
import ast
import hashlib
import json
import pathlib
import shutil
import sys

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent


def main(ref):
    ref = pathlib.Path(ref)
    files = {
        "test0.fits": ref / "res" / "test0.fits",
        "test1.fits": ref / "res" / "test1.fits",
        "test01_conv.fits": ref / "tests" / "test01_conv.fits",
        "test01_sub.fits": ref / "tests" / "test01_sub.fits",
    }
    manifest = {}
    for dst, src in files.items():
        shutil.copyfile(src, HERE / dst)
        manifest[dst] = {"source": str(src.relative_to(ref)),
                         "sha256": hashlib.sha256(src.read_bytes()).hexdigest()}
    txt = (ref / "tools" / "cond_num.py").read_text()
    start = txt.index("np.array(") + len("np.array(")
    end = txt.index("])", start) + 1
    mtx = np.array(ast.literal_eval(txt[start:end]), dtype=np.float64)
    assert mtx.shape == (293, 293)
    np.save(HERE / "test01_ksc_matrix.npy", mtx)
    manifest["test01_ksc_matrix.npy"] = {"source": "tools/cond_num.py:3-298",
                                         "shape": list(mtx.shape)}
    (HERE / "manifest.json").write_text(json.dumps(manifest, indent=1) + "\n")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_fixtures.py <path to the Thesis-EMX-BACH checkout>")
    main(sys.argv[1])
