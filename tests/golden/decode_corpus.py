"""Seeded corpus of POST /nearest bodies for the decode tests: numbers as
printf / repr / add_vectors.sh would write them (up to 17 significant
digits, exponents to the subnormal and overflow ends), whitespace of every
byte <= 32, objects, trailing content, and malformed or non-numeric bodies
for each of the handler's error branches (src/compare_handler.c:300-390)."""
from __future__ import annotations

import numpy as np


def number_texts(rng, n: int) -> list[bytes]:
    out = []
    for _ in range(n):
        u = rng.random()
        x = rng.normal() * 10.0 ** int(rng.integers(-5, 6))
        if u < 0.2:
            t = repr(float(x))
        elif u < 0.35:
            t = "%.17g" % x
        elif u < 0.45:
            t = "%.15g" % x
        elif u < 0.55:
            t = "%f" % x
        elif u < 0.65:  # test/add_vectors.sh: 1..9 and 0-6 decimals
            nd = int(rng.integers(0, 7))
            t = str(int(rng.integers(1, 10))) + ("." + "".join(str(d) for d in rng.integers(0, 10, nd)) if nd else "")
        elif u < 0.72:
            t = "%.17e" % (rng.normal() * 10.0 ** int(rng.integers(-300, 300)))
        elif u < 0.76:
            t = "%de%d" % (int(rng.integers(1, 10**6)), int(rng.integers(-345, -300)))  # subnormals and underflow
        elif u < 0.79:
            t = "%de%d" % (int(rng.integers(1, 10**6)), int(rng.integers(300, 320)))  # near and past overflow
        elif u < 0.82:
            t = "".join(str(d) for d in rng.integers(0, 10, int(rng.integers(18, 30)))) + "e-" + str(int(rng.integers(0, 40)))
        elif u < 0.85:
            t = "0.000" + "".join(str(d) for d in rng.integers(0, 10, 17))
        elif u < 0.88:
            t = "-0" if rng.random() < 0.5 else "-0.0e5"
        elif u < 0.91:
            t = "%.0f." % abs(x)  # "12." (strtod takes the point)
        elif u < 0.94:
            t = "-.%d" % int(rng.integers(0, 10**6))  # cJSON reads "-.5" though JSON would not
        elif u < 0.97:
            t = "%dE+%02d" % (int(rng.integers(0, 10**9)), int(rng.integers(0, 30)))
        else:
            t = "000%d.%d" % (int(rng.integers(0, 1000)), int(rng.integers(0, 1000)))
        out.append(t.encode())
    return out


def bodies(seed: int = 0, n: int = 2000, dim: int = 16) -> list[bytes]:
    rng = np.random.default_rng(seed)
    ws = [b" ", b"\n", b"\t", b"\r", b"", b"  \x01", b"\x1f"]
    out = []
    for i in range(n):
        nums = number_texts(rng, dim)
        w = lambda: ws[int(rng.integers(0, len(ws)))]
        kind = rng.random()
        if kind < 0.70:
            b = w() + b"[" + b",".join(w() + t + w() for t in nums) + b"]" + w()
        elif kind < 0.74:
            b = b"{" + b",".join(b'"k%d":' % j + t for j, t in enumerate(nums)) + b"}"  # counts like an array
        elif kind < 0.77:
            b = b"\xef\xbb\xbf[" + b",".join(nums) + b"] trailing {"  # BOM; content after the value ignored
        elif kind < 0.80:
            b = b"[" + b",".join(nums[:-1]) + b"]"  # size mismatch
        elif kind < 0.83:
            b = b"[" + b",".join(nums + [b"1"]) + b"]"
        elif kind < 0.86:
            j = int(rng.integers(0, dim))
            nums[j] = [b'"1.5"', b"null", b"true", b"[1]", b'{"a":1}', b'"\\u00e9\\n"'][int(rng.integers(0, 6))]
            b = b"[" + b",".join(nums) + b"]"  # invalid vector data
        elif kind < 0.89:
            b = b"[" + b",".join(nums) + [b"", b",", b" ,]", b"]]"][int(rng.integers(0, 4))]  # truncated / extra
        elif kind < 0.92:
            j = int(rng.integers(0, dim))
            nums[j] = [b"1e", b"1.5.3", b"+1", b"--1", b"0x10", b"1e+", b"inf", b"NaN", b"."][int(rng.integers(0, 9))]
            b = b"[" + b",".join(nums) + b"]"
        elif kind < 0.94:
            b = [b"", b"   ", b"5", b'"s"', b"null", b"[]", b"{}", b"[1,,2]", b"[1 2]"][int(rng.integers(0, 9))]
        elif kind < 0.96:
            b = b"[" + b",".join(nums) + b"]\x00" + b"garbage"  # a NUL ends the text
        elif kind < 0.98:
            j = int(rng.integers(0, dim))
            nums[j] = [b'"\\ud83d\\ude00"', b'"\\ud83d"', b'"\\ude00"', b'"\\x"', b'"\\uZZZZ"'][int(rng.integers(0, 5))]
            b = b"[" + b",".join(nums) + b"]"
        else:
            depth = int(rng.integers(990, 1010))
            b = b"[" + b"[" * depth + b"]" * depth + b"," + b",".join(nums[1:]) + b"]"  # nesting limit
        out.append(b)
    return out
