"""Extract the central rows of the Bickley finite-difference table.

Reads the DATA statements of BLOCK DATA BLKDS in the reference's
src/mates.f (COMMON /SDERA/ A(25792), layout unpacked by NEWDER ICON=1,
newder.f:84-127) and writes, for every odd M = 3..25 and derivative order
K = 1, 2, the M weights of the central row as the table's 25-digit decimal
strings.  Run where the reference is checked out (the path defaults to
$EP_REFERENCE_ROOT/src/mates.f, else to a "reference" directory beside this
repository):

    python tests/golden/make_fd_fixture.py [path/to/src/mates.f]
"""
import json
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def parse(path):
    lines = open(path, encoding="latin-1").read().splitlines()
    start = next(i for i, l in enumerate(lines) if "BLOCK DATA BLKDS" in l)
    A = {}
    i = start
    hdr = re.compile(r"DATA \(A\(I\),I=\s*(\d+),\s*(\d+)\)/")
    while i < len(lines):
        l = lines[i]
        if l.strip() == "END":
            break
        m = hdr.search(l)
        if m:
            a, b = int(m.group(1)), int(m.group(2))
            vals = []
            i += 1
            while len(vals) < b - a + 1:
                body = lines[i][6:]
                vals += [t for t in re.split(r"[,/\s]+", body.strip()) if t]
                i += 1
            for k, v in enumerate(vals[: b - a + 1]):
                A[a + k] = v.replace("D", "E")
            continue
        i += 1
    return A


def central_row(A, M, K):
    """Central row of the M x M matrix of order K (newder.f:84-110)."""
    ji = 1
    for I in range(3, M - 1, 2):
        ji += (I * I + 1) * (I - 2) // 2 + I
    m21o2 = (M * M + 1) // 2
    ji += m21o2 * (K - 1)
    sig = -1 if K % 2 else 1
    half = (M - 1) // 2
    first = [A[ji + half * M + j] for j in range(half + 1)]  # columns 1..half+1
    row = list(first)
    for j in range(half + 2, M + 1):  # columns half+2..M by symmetry
        v = first[M + 1 - j - 1]
        if sig < 0:
            v = v[1:] if v.startswith("-") else "-" + v.lstrip("+")
        row.append(v)
    return row


def main():
    root = os.environ.get("EP_REFERENCE_ROOT") or os.path.join(os.path.dirname(os.path.dirname(HERE)), "..",
                                                                "reference")
    path = sys.argv[1] if len(sys.argv) > 1 else os.path.join(root, "src", "mates.f")
    A = parse(path)
    out = {}
    for M in range(3, 26, 2):
        for K in (1, 2):
            if K >= M - 1:
                continue
            out[f"M{M}_K{K}"] = central_row(A, M, K)
    dst = os.path.join(HERE, "bickley_central_rows.json")
    with open(dst, "w") as f:
        json.dump({"source": "reference src/mates.f BLOCK DATA BLKDS (COMMON /SDERA/)",
                   "rows": out}, f, indent=1)
    print(dst, len(out))


if __name__ == "__main__":
    main()
