"""Generate tests/golden/dltc_tables.json: the DLTC residual tables as the
reference's own sources define them (DLTC/ccd-t2.cc, DLTC/ccsd-t1.cc,
DLTC/ccsd-t2.cc), read as text.

For each table: its tensors (enum order, index types HOL/PAR of their
Tensor2/Tensor4 constructors), every Multiplication m[i] and Summation s[i]
with the index names that setIndexName2/4 gave each operand just before it
(the constructor copies the tensor, so the names at that point are the
ones the expression keeps), its coefficient, and the dependency layers (the
exec(MUL|SUM, i) calls between Barrier()s).  tests/test_dltc_tables.py
checks the library's restated tables against this file.

Run from the repository root where the reference tree is present:
    python tests/golden/make_dltc_tables.py [path-to-DTCF-tree]
(default: $DTCF_REFERENCE, else /root/reference).
"""
import json
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
TABLES = {"ccd_t2": "DLTC/ccd-t2.cc", "ccsd_t1": "DLTC/ccsd-t1.cc", "ccsd_t2": "DLTC/ccsd-t2.cc"}
NAMES = ["h%d" % i for i in range(1, 13)] + ["p%d" % i for i in range(1, 13)]  # IndexName, DLTC/param.h


def parse(text):
    enum = re.search(r"enum\s+TensorName\s*\{([^}]*)\}", text).group(1)
    tensors = [t.strip() for t in enum.replace("\n", " ").split(",") if t.strip()]
    types = {}
    for m in re.finditer(r"T\[(\w+)\]\s*=\s*Tensor[24]\(([^)]*)\)", text):
        args = [a.strip() for a in m.group(2).split(",")]
        types[m.group(1)] = [a for a in args[:-1]]
    ids = {}
    muls, sums = {}, {}
    for line in text.splitlines():
        m = re.search(r"setIndexName[24]\(T\[(\w+)\],\s*([^)]*)\)", line)
        if m:
            ids[m.group(1)] = [NAMES.index(x.strip()) for x in m.group(2).split(",")]
            continue
        m = re.search(r"m\[(\d+)\]\s*=\s*Multiplication\(T\[(\w+)\],\s*T\[(\w+)\],\s*T\[(\w+)\],\s*([-+0-9.eE]+)\)", line)
        if m:
            i, c, a, b, coef = int(m.group(1)), m.group(2), m.group(3), m.group(4), float(m.group(5))
            muls[i] = dict(index=i, C=c, A=a, B=b, idC=ids[c], idA=ids[a], idB=ids[b], coef=coef)
            continue
        m = re.search(r"s\[(\d+)\]\s*=\s*Summation\(T\[(\w+)\],\s*T\[(\w+)\],\s*([-+0-9.eE]+)\)", line)
        if m:
            i, c, a, coef = int(m.group(1)), m.group(2), m.group(3), float(m.group(4))
            sums[i] = dict(index=i, C=c, A=a, idC=ids[c], idA=ids[a], coef=coef)
    layers, cur = [], None
    for line in text.splitlines():
        if re.search(r"TaskPool\s+tp\d+\s*=", line):
            cur = []
            layers.append(cur)
            continue
        m = re.search(r"exec\((MUL|SUM),\s*(\d+),", line)
        if m and cur is not None:
            cur.append([m.group(1), int(m.group(2))])
    return dict(tensors=tensors, types={t: types[t] for t in tensors}, muls=[muls[i] for i in sorted(muls)],
                sums=[sums[i] for i in sorted(sums)], layers=layers)


def main():
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("DTCF_REFERENCE", "/root/reference")
    out = {}
    for name, rel in TABLES.items():
        out[name] = parse(open(os.path.join(ref, rel)).read())
        out[name]["source"] = rel
    path = os.path.join(HERE, "dltc_tables.json")
    with open(path, "w") as f:
        json.dump(out, f, indent=1)
    for name, t in out.items():
        print(name, len(t["tensors"]), "tensors,", len(t["muls"]), "muls,", len(t["sums"]), "sums,",
              [len(l) for l in t["layers"]], "per layer")


if __name__ == "__main__":
    main()
