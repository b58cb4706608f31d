"""Golden bytes for the result writers: the reference C++ engine's own output
files of ``data/cpp_test_run`` (am_topopt --resolution 4 --iterations 5):
density_field.npy (cpp_engine/src/am_topopt.cpp:344-396), metadata.json
(:401-447) and history.csv (:622-629), stored verbatim.

    python tests/golden/make_writer_golden.py [/path/to/reference]
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def main(ref):
    run = os.path.join(ref, "data", "cpp_test_run")
    out = {}
    for key, name in (("npy", "density_field.npy"), ("metadata", "metadata.json"), ("history", "history.csv")):
        with open(os.path.join(run, name), "rb") as f:
            out[key] = np.frombuffer(f.read(), dtype=np.uint8)
    np.savez_compressed(os.path.join(HERE, "writer_golden.npz"), **out)
    print("wrote", os.path.join(HERE, "writer_golden.npz"))


if __name__ == "__main__":
    if len(sys.argv) != 2:
        raise SystemExit(f"usage: python {sys.argv[0]} <path of the reference checkout>")
    main(sys.argv[1])
