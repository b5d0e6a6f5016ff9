"""Generates the golden fixtures in tests/golden/ from the reference's own
host code.

Runs in the build container, where the reference sources are mounted.  For
each configuration it compiles the reference's host functions (main.cu,
GPU.cu, kernel.cu, import_dataset.cpp, par_sort.cpp) through
oracle/build_ref_host.sh, feeds them seeded inputs through
oracle/ref_host_driver.cpp, and stores inputs and outputs here:

  prep_<tag>.npz   ReorderByDimension (main.cu:2521), generateNDGridDimensions
                   (main.cu:2425), populateNDGridIndexAndLookupArrayParallel
                   (main.cu:1968) and computeWorkDifficulty (main.cu:2941)
  csv_<tag>.npz    importNDDataset (import_dataset.cpp:50) on csv_input.csv
  print_*.txt      printNeighborTable (main.cu:911) and printOutlierScores
                   (main.cu:952) on a table from print_input.npz

usage: python tests/golden/make_golden.py [REFDIR]
"""
from __future__ import annotations

import os
import struct
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402

REFDIR = sys.argv[1] if len(sys.argv) > 1 else "/root/reference"

# (dtype, GPUNUMDIM, NUMINDEXEDDIM, n, generator)
CONFIGS = [
    ("float", 2, 2, 3000, "clumps2d"),
    ("double", 6, 6, 2000, "gmm6d"),
    ("float", 5, 3, 2500, "aniso5d"),
]


def gen(kind: str, n: int, d: int, dtype) -> np.ndarray:
    rng = np.random.default_rng({"clumps2d": 11, "gmm6d": 12, "aniso5d": 13}[kind])
    if kind == "clumps2d":
        x = np.empty((n, 2))
        x[:, 0] = rng.uniform(0, 360, n)
        x[:, 1] = rng.normal(0, 8, n).clip(-90, 90)
        c = rng.integers(0, n, 10)
        for i, ci in enumerate(c):
            sl = slice(i * 50, i * 50 + 50)
            x[sl] = x[ci] + rng.normal(0, 0.2, (50, 2))
        x[2000:2010] = x[5]  # exact duplicates
    elif kind == "gmm6d":
        centers = rng.random((8, d))
        lab = rng.integers(0, 8, n)
        x = centers[lab] + rng.normal(0, 1, (n, d)) * rng.uniform(0.005, 0.1, (8, d))[lab]
        x[: n // 10] = rng.random((n // 10, d))
    else:
        x = rng.normal(0, 1, (n, d)) * np.array([0.5, 3.0, 1.0, 0.1, 2.0])
    return np.ascontiguousarray(x.astype(dtype))


def write_points(path: str, x: np.ndarray) -> None:
    with open(path, "wb") as f:
        f.write(struct.pack("<QI", x.shape[0], x.shape[1]))
        f.write(x.tobytes())


CSV_TEXT = (
    "1.5,2.25\n"
    "3,4\r\n"
    " 5.125 , -6.5\n"
    "7e-3,+8.0\n"
    "\n"
    "9.75,1e2,\n"
    "0.1,0.2\n"
    "12abc,13\n"
    "14,15\n"
    ".5,6.\n"
    "16 17,18\n"
    "19,20,21"
)


def main() -> None:
    out_files = []
    with tempfile.TemporaryDirectory() as tmp:
        for dtype, ndim, nidx, n, kind in CONFIGS:
            tag = f"{dtype}_{ndim}_{nidx}"
            drv = subprocess.check_output(
                ["bash", os.path.join(ROOT, "oracle", "build_ref_host.sh"), dtype, str(ndim),
                 str(nidx), REFDIR], text=True).strip().splitlines()[-1]
            npdt = np.float32 if dtype == "float" else np.float64
            x = gen(kind, n, ndim, npdt)
            inp = os.path.join(tmp, f"in_{tag}.bin")
            write_points(inp, x)
            perm, _ = oracle.reorder(x)
            est = oracle.estimate_eps(x[:, perm], k=8, beta=0.05)
            eps = float(npdt(est["eps0"]))
            pre = os.path.join(tmp, f"o_{tag}_")
            subprocess.check_call([drv, "prep", inp, repr(eps), pre])

            def rd(name, dt):
                return np.fromfile(pre + name + ".bin", dt)

            np.savez_compressed(
                os.path.join(HERE, f"prep_{tag}.npz"),
                data=x, eps=np.array(eps, npdt), num_indexed_dims=np.array(nidx),
                reordered=rd("reordered", npdt).reshape(n, ndim),
                minArr=rd("minArr", npdt), maxArr=rd("maxArr", npdt),
                nCells=rd("nCells", np.uint32), totalCells=rd("totalCells", np.uint64),
                cellKeys=rd("cellKeys", np.uint64), cellIdx=rd("cellIdx", np.uint32),
                indexmin=rd("indexmin", np.int32), indexmax=rd("indexmax", np.int32),
                lookup=rd("lookup", np.uint32), workorder=rd("workorder", np.uint32),
            )
            out_files.append(f"prep_{tag}.npz")

            if ndim == 2:
                # CSV import through the same build (GPUNUMDIM=2)
                csv_path = os.path.join(HERE, "csv_input.csv")
                with open(csv_path, "w", newline="") as f:
                    f.write(CSV_TEXT)
                ob = os.path.join(tmp, "csv.bin")
                subprocess.check_call([drv, "csv", csv_path, ob])
                raw = open(ob, "rb").read()
                npts = struct.unpack("<Q", raw[:8])[0]
                vals = np.frombuffer(raw[8:], npdt).reshape(npts, ndim)
                np.savez_compressed(os.path.join(HERE, f"csv_{tag}.npz"), points=vals)
                out_files.append(f"csv_{tag}.npz")

                # KNN_out / outlier-score text from a small oracle table
                xs = gen("clumps2d", 3000, 2, np.float32)[:1500].copy()
                rc, ids, dists, _ = oracle.join(xs, 4, di=2, beta=0.05)
                assert rc == 0
                np.savez_compressed(os.path.join(HERE, "print_input.npz"), data=xs, ids=ids,
                                    dists=dists)
                tb = os.path.join(tmp, "table.bin")
                with open(tb, "wb") as f:
                    f.write(struct.pack("<QI", ids.shape[0], ids.shape[1]))
                    f.write(ids.astype(np.int32).tobytes())
                    f.write(dists.astype(np.float32).tobytes())
                od = os.path.join(tmp, "print")
                os.makedirs(od)
                subprocess.check_call([drv, "print", tb, od])
                for name in ("KNN_out.txt", "KNN_out_distances.txt", "KNN_outlier_scores.txt"):
                    with open(os.path.join(od, name)) as fi, open(
                            os.path.join(HERE, "print_" + name), "w") as fo:
                        fo.write(fi.read())
                    out_files.append("print_" + name)
    print("wrote", ", ".join(out_files))


if __name__ == "__main__":
    main()
