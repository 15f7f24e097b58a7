"""OBJ inputs for the loader tests (load_obj, mesh.rs:474-642): hand-written
edge cases, a seeded generator of irregular files, decimals that sit on or near
binary32 rounding boundaries, and an exact decimal -> binary32 rounding in
rational arithmetic (the value str::parse::<f32> must return)."""
from fractions import Fraction
import random
import re

import numpy as np

EDGE_CASES = {
    "shared_normals": b"v 0 0 0\nv 1 0 0\nv 0 1 0\nv 1 1 0\nvn 0 0 1\nf 1//1 2//1 3//1\nf 2//1 4//1 3//1\n",
    "no_normals_polygons": b"v 0 0 0\nv 1 0 0\nv 1 1 0\nv 0 1 0\nv -1 0.5 0\nf 1 2 3 4\nf 1 2 3 4 5\nf 3 2 1\n",
    "negative_indices": b"v 0 0 0\nv 1 0 0\nv 0 1 0\nvn 0 0 -1\nf -3//-1 -2//-1 -1//1\nv 2 2 2\nf -1 -2 -3\n",
    "forward_and_bad_refs": b"f 1 2 3\nv 0 0 0\nv 1 0 0\nf 1 2 5\nf 0 -0 +1\nf 1//7 2//1 1//\nvn 1 0 0\n"
                            b"f 1//1 2//2 1//99\n",
    "part_forms": b"v 0 0 0\nv 1 0 0\nv 0 1 0\nvt 0.25 0.75\nvn 0 1 0\n"
                  b"f 1/ 2/1 3/1/\nf 1//1 2/1/1 3/1/1/7\nf //1 /1/1 3\nf 1/2 2/1 3/-1\n",
    "whitespace": b"  v\t0 0 0 \r\nv 1\x0c0 0\r\n\tv 0 1 0\x0b\r\n\x0bvn 0 0 1\nf 1//1\t2//1   3//1  \r\n"
                  b"v\x0b1 2 3\n   \n\t\n",
    "comments": b"# header\nv 0 0 0\n   # indented comment\nv 1 0 0 # trailing\nv 0 1 0\n"
                b"f 1 2 3 # a comment is three more tokens\n#f 1 2 3\n",
    "component_counts": b"v 1 2\nv 0 0 0 1\nv 1 0 0 0.5\nv 0 1 0\nvt 0.5\nvt 0.1 0.2 0.3\nvn 0 0 0\nvn 3 4 0\n"
                        b"f 1 2\nf 1/1/1 2/1/2 3/1/1\n",
    "float_forms": b"v 1e0 1E-3 +2.5\nv .5 5. -.5e+1\nv inf -Infinity NaN\nv nan -nan INF\n"
                   b"v 1.5f 0x10 1_0\nv --1 1e e5\nv 1e+ . -\nf 1 2 3\nf 4 5 6 7\n",
    "index_forms": b"v 0 0 0\nv 1 0 0\nv 0 1 0\nvn 0 0 1\n"
                   b"f +1//+1 2//1 3//1\nf 99999999999999999999 2 3\nf -9223372036854775808 1 2\n"
                   b"f 1.0 2 3\nf 1//1 2//1 3//1.0\nf 1//99999999999999999999 2//1 3//1\n",
    "unicode_trim": "v 0 0 0 \nv 1 0 0　\n v 0 1 0\nv 0 1 0\n﻿v 9 9 9\n"
                    "vn 0 0 1 \nf 1//1 2//1 3//1 \n# café 中\n".encode(),
    "no_trailing_newline": b"v 0 0 0\nv 1 0 0\nv 0 1 0\nf 1 2 3",
    "uv_keys": b"v 0 0 0\nv 1 0 0\nv 0 1 0\nvt 0 0\nvt 1 1\nvn 0 0 1\n"
               b"f 1/1/1 2/1/1 3/1/1\nf 1/2/1 2/1/1 3/2/1\nf 1/1/1 2/2/1 3/1/1\nf 1/1 2/2 3/1\n",
    "mixed_has_norm_fan": b"v 0 0 0\nv 1 0 0\nv 1 1 0\nv 0 1 0\nv -1 1 0\nvn 0 0 1\n"
                          b"f 1 2//1 3 4//1 5\nf 1//1 2 3//1 4\n",
    "degenerate": b"v 0 0 0\nv 1 1 1\nv 2 2 2\nv 0 0 0\nf 1 2 3\nf 1 4 1\n",
    "nan_positions": b"v nan 0 0\nv 1 0 0\nv 0 1 0\nf 1 2 3\n",
    "extreme_decimals": b"v 1e-46 1e-45 7.006492321624085e-46\nv 3.4028235e38 3.4028236e38 3.40282356e38\n"
                        b"v 1e39 -1e39 1e-400\nv 16777217 16777219 0.1\n"
                        b"v 1.00000000000000000000000000000000000000000000000001 0.333333333333333333333333333 "
                        b"-0.000000000000000000000000000000000000000000001401298464324817\n"
                        b"v 0.0000000000000000000000000000000000000000000007006492321624085354618647916449580656401309709382578858785341419448955413429303 "
                        b"0.00000000000000000000000000000000000000000000070064923216240853546186479164495806564013097093825788587853414194489554134293031 "
                        b"1e99999\nf 1 2 3\nf 4 5 6\n",
}

# (name, text, expected error text after "'<path>' " / "'<path>': ")
ERROR_CASES = [
    ("empty", b"", "no geometry found after parsing"),
    ("vertices_only", b"v 0 0 0\nv 1 0 0\nv 0 1 0\n", "no geometry found after parsing"),
    ("two_token_face", b"v 0 0 0\nv 1 0 0\nf 1 2\n", "no geometry found after parsing"),
    ("lone_continuation", b"v 0 0 0\n\x80\nf 1 1 1\n",
     "is not valid UTF-8: invalid utf-8 sequence of 1 bytes from index 8"),
    ("truncated_at_end", b"v 0 0 0\nf 1 1 1\n\xe2\x82", "is not valid UTF-8: incomplete utf-8 byte sequence from index 16"),
    ("overlong", b"v 0 0 0\xc0\x80\n", "is not valid UTF-8: invalid utf-8 sequence of 1 bytes from index 7"),
    ("surrogate", b"f 1 1 1\n\xed\xa0\x80", "is not valid UTF-8: invalid utf-8 sequence of 1 bytes from index 8"),
    ("bad_third_byte", b"v \xe2\x82\x28 0 0\n", "is not valid UTF-8: invalid utf-8 sequence of 2 bytes from index 2"),
    ("bad_fourth_byte", b"# \xf0\x9f\x98\x41\n", "is not valid UTF-8: invalid utf-8 sequence of 3 bytes from index 2"),
    ("f5_lead", b"v 0 0 0\n\xf5\x80\x80\x80\n", "is not valid UTF-8: invalid utf-8 sequence of 1 bytes from index 8"),
    ("extra_continuation", b"v \xc3\xa9\xa9\n", "is not valid UTF-8: invalid utf-8 sequence of 1 bytes from index 4"),
]

HARD_DECIMALS = [
    "16777217", "16777219", "16777218.999999999999999999", "16777217.000000000000000001", "33554435",
    "0.1", "0.2", "0.3", "1.1", "3.14159265358979323846264338327950288", "2.7182818284590452353602874713527",
    "1e-45", "1.4e-45", "7e-46", "7.006492321624085e-46", "7.006492321624086e-46", "1.401298464324817e-45",
    "2.1019476964872256e-45", "2.1019476964872257e-45", "1.1754942e-38", "1.17549435e-38", "1.1754943508222875e-38",
    "1.1754942807573643e-38", "1.1754942807573644e-38", "3.4028234663852886e38", "3.4028235677973366e38",
    "3.4028235677973367e38", "3.4028235677973365e38", "340282356779733661637539395458142568448",
    "340282356779733661637539395458142568447", "4.9406564584124654e-324", "1e38", "9.999999e37", "123456789",
    "1234567891", "8388609.5", "8388608.5", "0.000000059604644775390625", "0.0000000596046447753906250000000001",
    "1.00000005960464477539062499999999", "1.000000059604644775390625", "1.00000017881393432617187500000000001",
    "99999999999999999999999999999", "0.999999999999999999999999999999999999999", "5e-324", "2.5e-45",
    "12345678901234567890123456789e-20", "-0", "-0.0", "+0e10", "0e-999999", "1" + "0" * 60, "0." + "0" * 50 + "1",
]


def exact_f32_bits(text):
    """uint32 bits of the binary32 nearest to the decimal (ties to even), or
    None if the text is not Rust f32 syntax.  Rational arithmetic only."""
    m = re.fullmatch(r"([+-]?)(\d*)(?:\.(\d*))?(?:[eE]([+-]?\d+))?", text)
    low = text.lower().lstrip("+-")
    neg = text.startswith("-")
    if low in ("inf", "infinity"):
        return 0xFF800000 if neg else 0x7F800000
    if low == "nan":
        return 0xFFC00000 if neg else 0x7FC00000
    if not m or not (m.group(2) or m.group(3)):
        return None
    digits = (m.group(2) or "") + (m.group(3) or "")
    exp = int(m.group(4) or 0) - len(m.group(3) or "")
    if exp > 400:
        exp = 400 if int(digits or "0") else 0
    if exp < -100000:
        exp = -100000
    x = Fraction(int(digits or "0")) * (Fraction(10) ** exp if exp >= 0 else Fraction(1, 10 ** -exp))
    sign = 0x80000000 if neg else 0
    if x == 0:
        return sign
    e = x.numerator.bit_length() - x.denominator.bit_length()
    if Fraction(2) ** e > x:
        e -= 1
    ulp_e = max(e, -126) - 23
    q = x / (Fraction(2) ** ulp_e)
    k = q.numerator // q.denominator
    r = q - k
    if r > Fraction(1, 2) or (r == Fraction(1, 2) and k % 2 == 1):
        k += 1
    v = Fraction(k) * Fraction(2) ** ulp_e
    if v >= Fraction(2) ** 128:
        return sign | 0x7F800000
    return sign | int(np.array(float(v), np.float32).view(np.uint32))


_NUMS = ["0", "1", "-1", "0.5", "-2.25", "1e3", "-1.5e-2", ".25", "3.", "+4", "1.0000001", "123456.789",
         "0.1", "nan", "inf", "-inf", "1e-40", "3e38", "bad", "1.2.3", "--2", "", "7e", "0x1"]


def random_obj(seed, n_lines=400):
    """A seeded irregular OBJ file: every directive kind, index forms (relative,
    absolute, out of range, malformed), token forms, numbers (good and bad),
    CRLF, tabs, comments, blank lines and unknown directives."""
    rng = np.random.default_rng(seed)
    out = []
    nv = nvt = nvn = 0
    def num():
        r = rng.random()
        if r < 0.7:
            return f"{rng.normal() * 3:.{int(rng.integers(0, 9))}f}"
        if r < 0.85:
            return f"{rng.normal():.7e}"
        return _NUMS[int(rng.integers(len(_NUMS)))]
    def idx(n):
        r = rng.random()
        if r < 0.6 and n:
            return str(int(rng.integers(1, n + 1)))
        if r < 0.8 and n:
            return str(-int(rng.integers(1, n + 1)))
        return ["0", "-0", str(n + 3), "x", "", "+1", "99999999999999999999", "1.5"][int(rng.integers(8))]
    for _ in range(n_lines):
        r = rng.random()
        ws = " " if rng.random() < 0.8 else ["\t", "  ", " \t "][int(rng.integers(3))]
        if r < 0.3:
            k = int(rng.choice([3, 3, 3, 4, 2]))
            out.append("v" + "".join(ws + num() for _ in range(k)))
            nv += k >= 3
        elif r < 0.42:
            out.append("vn" + "".join(ws + num() for _ in range(3)))
            nvn += 1
        elif r < 0.5:
            k = int(rng.choice([2, 2, 3, 1]))
            out.append("vt" + "".join(ws + num() for _ in range(k)))
            nvt += k >= 2
        elif r < 0.85:
            n_tok = int(rng.choice([3, 3, 3, 4, 5, 6, 2]))
            form = int(rng.integers(6))
            toks = []
            for _ in range(n_tok):
                f = form if rng.random() < 0.85 else int(rng.integers(6))
                a, b, c = idx(nv), idx(nvt), idx(nvn)
                toks.append([a, f"{a}/{b}", f"{a}//{c}", f"{a}/{b}/{c}", f"{a}/", f"{a}/{b}/{c}/1"][f])
            out.append("f" + "".join(ws + t for t in toks))
        elif r < 0.9:
            out.append(["# comment v 1 2 3", "", "   ", "o object", "g group", "s 1", "usemtl m", "vp 1 2"][
                int(rng.integers(8))])
        else:
            out.append(ws + "f" + ws + " ".join(idx(nv) for _ in range(3)) + ws)
    eol = "\r\n" if rng.random() < 0.3 else "\n"
    return (eol.join(out) + (eol if rng.random() < 0.7 else "")).encode()


def mutated_obj(seed):
    """An edge-case or seeded random file with 1..6 byte-level edits drawn from
    the characters OBJ text is made of (inserted, replaced, deleted, or a
    run duplicated): near-valid text that exercises the loader's error paths
    and its tokenising next to them."""
    rng = random.Random(seed)
    seeds = [EDGE_CASES[k] for k in sorted(EDGE_CASES)]
    text = bytearray(rng.choice(seeds) if rng.random() < 0.5 else random_obj(rng.randrange(6)))
    alphabet = b" /\n\r\t0123456789-+.eEfvtn#"
    for _ in range(rng.randint(1, 6)):
        op = rng.random()
        if op < 0.25 and text:
            text[rng.randrange(len(text))] = rng.choice(alphabet)
        elif op < 0.45 and text:
            del text[rng.randrange(len(text))]
        elif op < 0.75:
            text.insert(rng.randrange(len(text) + 1), rng.choice(alphabet))
        elif text:
            i = rng.randrange(len(text))
            text[i:i] = text[i:min(len(text), i + rng.randint(1, 40))]
    return bytes(text)


def canon(v):
    """Vertex records as uint32 words with every NaN mapped to one pattern (NaN
    payloads differ between CPU and GPU arithmetic)."""
    f = np.ascontiguousarray(v).view(np.float32).reshape(len(v), -1)
    w = f.view(np.uint32).copy()
    w[np.isnan(f)] = 0x7FC00000
    return w
