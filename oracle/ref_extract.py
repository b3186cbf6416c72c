"""Build step of the reference library (test infrastructure only): writes the
definitions of nscale's own CPU functions on the segmentNuclei path, taken
verbatim from the nscale sources at build time, into one include file under
oracle/_ref/ (git-ignored).  oracle/ref_nscale_wrap.cpp compiles them against
oracle/cvstandin/cv_standin.hpp, in place of OpenCV, so the oracle can be
checked against the reference's own code.  Nothing taken from the nscale
tree is written anywhere but oracle/_ref/.

Each function is located by its signature, extended back over its
`template <...>` line and forward to its matching closing brace (comments and
literals skipped); a #line directive keeps compiler messages pointing at the
nscale file.

usage: python ref_extract.py <nscale root> <output .inc>
"""
from __future__ import annotations

import os
import re
import sys

# (file under the nscale root, signature regex)
FUNCTIONS = [
    ("src/segment/PixelOperations.cpp", r"^\s*Mat PixelOperations::invert\(const Mat &img\)"),
    ("src/segment/MorphologicOperations.cpp", r"^inline void propagate\(const Mat& image, Mat& output"),
    ("src/segment/MorphologicOperations.cpp", r"^Mat imreconstruct\(const Mat& seeds, const Mat& image, int connectivity\)"),
    ("src/segment/MorphologicOperations.cpp", r"^inline void propagateBinary\(const Mat& image"),
    ("src/segment/MorphologicOperations.cpp", r"^Mat imreconstructBinary\(const Mat& seeds"),
    ("src/segment/MorphologicOperations.cpp", r"^Mat imfillHoles\(const Mat& image"),
    ("src/segment/MorphologicOperations.cpp", r"^Mat bwselect\(const Mat& binaryImage"),
    ("src/segment/MorphologicOperations.cpp", r"^Mat_<int> bwlabel2\(const Mat& binaryImage"),
    ("src/segment/MorphologicOperations.cpp", r"^Mat bwareaopen2\(const Mat& image"),
    ("src/segment/MorphologicOperations.cpp", r"^Mat imhmin\(const Mat& image"),
    ("src/segment/MorphologicOperations.cpp", r"^Mat_<unsigned char> localMaxima\(const Mat& image"),
    ("src/segment/MorphologicOperations.cpp", r"^Mat_<unsigned char> localMinima\(const Mat& image"),
    ("src/segment/MorphologicOperations.cpp", r"^Mat_<int> watershed2\(const Mat& origImage"),
    ("src/segment/MorphologicOperations.cpp", r"^Mat morphOpen\(const Mat& image, const Mat& kernel\)"),
    ("src/segment/NeighborOperations.cpp", r"^Mat NeighborOperations::border\(Mat& img"),
    ("src/segment/HistologicalEntities.cpp", r"^Mat HistologicalEntities::getRBC\(const std::vector<Mat>& bgr"),
    ("src/segment/HistologicalEntities.cpp", r"^Mat HistologicalEntities::getBackground\(const std::vector<Mat>& bgr"),
    ("src/segment/HistologicalEntities.cpp", r"^int HistologicalEntities::plFindNucleusCandidates\("),
    ("src/segment/HistologicalEntities.cpp", r"^int HistologicalEntities::plSeparateNuclei\("),
    ("src/segment/HistologicalEntities.cpp", r"^int HistologicalEntities::segmentNuclei\(const Mat& img, Mat& output,\s*$"),
    ("src/segment/HistologicalEntities.cpp",
     r"^int HistologicalEntities::segmentNuclei\(const Mat& img, Mat& output, unsigned char blue"),
]


def _body_end(lines: list[str], start: int) -> int:
    """Index of the line holding the brace that closes the first '{' at or
    after line `start` (comments, string and character literals skipped)."""
    depth, opened = 0, False
    in_block = False
    for i in range(start, len(lines)):
        s = lines[i]
        j = 0
        while j < len(s):
            c = s[j]
            if in_block:
                if s.startswith("*/", j):
                    in_block = False
                    j += 2
                    continue
                j += 1
                continue
            if s.startswith("//", j):
                break
            if s.startswith("/*", j):
                in_block = True
                j += 2
                continue
            if c in "\"'":
                k = j + 1
                while k < len(s) and s[k] != c:
                    k += 2 if s[k] == "\\" else 1
                j = k + 1
                continue
            if c == "{":
                depth += 1
                opened = True
            elif c == "}":
                depth -= 1
                if opened and depth == 0:
                    return i
            j += 1
    raise ValueError(f"no closing brace after line {start + 1}")


def extract(root: str, rel: str, pattern: str) -> tuple[int, list[str]]:
    path = os.path.join(root, rel)
    with open(path, encoding="latin-1") as f:
        lines = f.read().splitlines()
    rx = re.compile(pattern)
    hits = [i for i, ln in enumerate(lines) if rx.search(ln)]
    if len(hits) != 1:
        raise ValueError(f"{rel}: {len(hits)} matches for {pattern!r}")
    start = hits[0]
    k = start - 1
    while k >= 0 and not lines[k].strip():
        k -= 1
    if k >= 0 and lines[k].strip().startswith("template"):
        start = k
    end = _body_end(lines, hits[0])
    return start + 1, lines[start:end + 1]


def main(root: str, out: str) -> None:
    parts = []
    for rel, pattern in FUNCTIONS:
        first, body = extract(root, rel, pattern)
        parts.append(f'#line {first} "{rel}"')
        parts.extend(body)
        parts.append("")
    os.makedirs(os.path.dirname(os.path.abspath(out)), exist_ok=True)
    tmp = out + ".tmp"
    with open(tmp, "w") as f:
        f.write("\n".join(parts) + "\n")
    os.replace(tmp, out)


if __name__ == "__main__":
    main(sys.argv[1], sys.argv[2])
