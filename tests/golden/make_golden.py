"""Regenerate the golden fixtures in this folder from the reference's test data.

Reads (at generation time only) the reference checkout's
``testdata/6-gaussian-4d.csv`` (200 points, 4-d, loaded the way
src/outlier/common.rs:200-226 loads it) and the ELKI-generated
``testdata/reference-outlier-scores.csv`` (rows KNN-10 and LOF-10, compared by
src/outlier/knn.rs:78-96 and src/outlier/lof.rs:193-211 with abs tol 1e-6).

Usage:  python tests/golden/make_golden.py /path/to/reference
The committed JSON files are what the tests read; the reference checkout is
not needed at test time.
"""
import json
import os
import sys


def load_points(path):
    pts, labels = [], []
    with open(path) as fh:
        for line in fh:
            line = line.strip()
            if not line or line.startswith("#"):
                continue
            parts = line.split()
            if len(parts) < 5:
                continue
            pts.append([float(x) for x in parts[:4]])
            labels.append(parts[4])
    return pts, labels


def load_scores(path, names):
    out = {}
    with open(path) as fh:
        for line in fh:
            line = line.strip()
            if not line or line.startswith("#"):
                continue
            parts = line.split()
            if parts[0] in names:
                out[parts[0]] = [float(x) for x in parts[1:]]
    return out


def main(ref_root):
    here = os.path.dirname(os.path.abspath(__file__))
    pts, labels = load_points(os.path.join(ref_root, "testdata", "6-gaussian-4d.csv"))
    scores = load_scores(os.path.join(ref_root, "testdata", "reference-outlier-scores.csv"), {"KNN-10", "LOF-10"})
    with open(os.path.join(here, "gaussian4d.json"), "w") as fh:
        json.dump({"source": "testdata/6-gaussian-4d.csv", "points": pts, "labels": labels}, fh)
    with open(os.path.join(here, "outlier_scores.json"), "w") as fh:
        json.dump({"source": "testdata/reference-outlier-scores.csv", "k": 10, "tolerance": 1e-6, **scores}, fh)
    print("wrote", len(pts), "points and", sorted(scores))


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py <root of the fuel source tree>")
    main(sys.argv[1])
