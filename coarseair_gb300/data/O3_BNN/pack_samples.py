"""Pack the O3 BNN posterior samples of one parameter folder into one gzip file.

BNN_PES_Class.F90 reads, for sample s, CalibratedParams/<name>.csv.<s> for Lambda, re, W1 (6 rows of
NHL1), b1, W2 (NHL1 rows of NHL2), b2, W3, b3, Sigma and Noise (ReadParamPost_BNN), and the folder's
ScalingValues.csv.  This script writes one line per sample -- s, NHL1, NHL2, Lambda, re, Noise, b3,
W1 row by row, b1, W2 row by row, b2, W3 -- with the values as the files hold them, and copies
ScalingValues.csv.  Usage: python pack_samples.py <reference>/dtb/Systems/O3/PESs/BNN/<folder>
"""
import gzip
import os
import shutil
import sys


def values(path):
    with open(path) as f:
        return [[x.strip() for x in ln.split(",")] for ln in f.read().splitlines() if ln.strip()]


def main(src):
    name = os.path.basename(os.path.normpath(src))
    here = os.path.dirname(os.path.abspath(__file__))
    cp = os.path.join(src, "CalibratedParams")
    samples = sorted({int(f.rsplit(".", 1)[1]) for f in os.listdir(cp) if f.startswith("W1.csv.")})
    lines = ["# sample,NHL1,NHL2,Lambda,re,Noise,b3,W1(6,NHL1) by rows,b1,W2(NHL1,NHL2) by rows,b2,W3"]
    for s in samples:
        get = lambda n: values(os.path.join(cp, "%s.csv.%d" % (n, s)))
        W1, W2 = get("W1"), get("W2")
        h1, h2 = len(W1[0]), len(W2[0])
        assert len(W1) == 6 and len(W2) == h1
        flat = [str(s), str(h1), str(h2), get("Lambda")[0][0], get("re")[0][0], get("Noise")[0][0], get("b3")[0][0]]
        flat += [x for row in W1 for x in row] + [r[0] for r in get("b1")]
        flat += [x for row in W2 for x in row] + [r[0] for r in get("b2")] + [r[0] for r in get("W3")]
        lines.append(",".join(flat))
    os.makedirs(os.path.join(here, name), exist_ok=True)
    with gzip.open(os.path.join(here, name, "samples.csv.gz"), "wt") as f:
        f.write("\n".join(lines) + "\n")
    shutil.copy(os.path.join(src, "ScalingValues.csv"), os.path.join(here, name, "ScalingValues.csv"))


if __name__ == "__main__":
    main(sys.argv[1])
