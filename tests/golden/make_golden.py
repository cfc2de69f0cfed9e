"""Generate the golden fixtures under tests/golden/ from the reference sources.

Run once, in a container that has the reference checked out:

    python tests/golden/make_golden.py <path of the reference checkout>

It reads three reference files as text and writes:

* ``kat.json`` -- the known-answer vectors of ``lib/src/test_data.rs:15-135``
  (eight single-block datasets: encoded bytes + decoded RGBA8), the odd-height
  BC1 decode case of ``lib/src/lib.rs:416-444`` and the storage-size cases of
  ``lib/src/lib.rs:350-361``.
* ``single_lut_sha256.json`` -- a SHA-256 of each single-colour lookup table of
  ``lib/src/colourfit/single_lut.rs`` (256 rows x 6 bytes, row-major
  start0,end0,err0,start1,end1,err1).  The tables themselves are not stored:
  both the oracle and the CUDA library regenerate them, and the tests compare
  the regenerated bytes against these digests.

The decoded images of ``test_data.rs`` are written there as calls to two const
helpers (``expand_single_to_rgb``, ``add_alpha_to_rgb``); this script evaluates
those calls with a tiny interpreter instead of copying expanded data.
"""
import hashlib
import json
import os
import re
import sys


def _byte_list(text):
    vals = []
    for tok in re.split(r"[,\s]+", text.strip()):
        if not tok:
            continue
        vals.append(int(tok, 0))
    return vals


def _strip_comments(src):
    return re.sub(r"//[^\n]*", "", src)


class _Eval:
    """Evaluates the const expressions used in lib/src/test_data.rs."""

    def __init__(self, src):
        self.src = _strip_comments(src)
        self.consts = {}
        for m in re.finditer(r"const\s+([A-Z0-9_]+)\s*:\s*\[u8;[^\]]*\]\s*=\s*\[(.*?)\];", self.src, re.S):
            self.consts[m.group(1)] = _byte_list(m.group(2))

    def expr(self, s):
        s = s.strip()
        if s.startswith("&"):
            return self.expr(s[1:])
        m = re.fullmatch(r"\[\s*(0x[0-9A-Fa-f]+|\d+)\s*;\s*(\d+)\s*\]", s)
        if m:
            return [int(m.group(1), 0)] * int(m.group(2))
        if s.startswith("[") and s.endswith("]"):
            return _byte_list(s[1:-1])
        if s in self.consts:
            return list(self.consts[s])
        m = re.fullmatch(r"([a-z_]+)\((.*)\)", s, re.S)
        if m:
            fn, args = m.group(1), self._split_args(m.group(2))
            vals = [self.expr(a) for a in args]
            if fn == "expand_single_to_rgb":
                (v,) = vals
                return [c for x in v for c in (x, x, x)]
            if fn == "add_alpha_to_rgb":
                rgb, alpha = vals
                out = []
                for i in range(16):
                    out += rgb[3 * i:3 * i + 3] + [alpha[i]]
                return out
        raise ValueError("cannot evaluate: %r" % s[:80])

    @staticmethod
    def _split_args(s):
        depth, cur, out = 0, "", []
        for ch in s:
            if ch in "([":
                depth += 1
            elif ch in ")]":
                depth -= 1
            if ch == "," and depth == 0:
                out.append(cur)
                cur = ""
            else:
                cur += ch
        if cur.strip():
            out.append(cur)
        return out

    def datasets(self):
        out = {}
        for m in re.finditer(r"pub const ([A-Z0-9_]+): TestDataSet = TestDataSet \{(.*?)\n\};", self.src, re.S):
            name, body = m.group(1), m.group(2)
            enc = re.search(r"encoded:\s*&\[(.*?)\],\s*decoded:", body, re.S).group(1)
            dec = body[body.index("decoded:") + len("decoded:"):].strip().rstrip(",")
            out[name] = {"encoded": _byte_list(enc), "decoded": self.expr(dec)}
        return out


def _lib_cases(lib_src):
    src = _strip_comments(lib_src)
    sizes = []
    for m in re.finditer(r"Format::(Bc\d)\.compressed_size\((\d+),\s*(\d+)\),\s*(\d+)\)", src):
        sizes.append({"format": m.group(1).upper(), "width": int(m.group(2)),
                      "height": int(m.group(3)), "size": int(m.group(4))})
    fn = src[src.index("fn test_bc1_decompression_height_not_multiple_of_4"):]
    enc = _byte_list(re.search(r"let encoded = \[(.*?)\];", fn, re.S).group(1))
    w, h = (int(x) for x in re.search(r"Format::Bc1\.decompress\(&encoded,\s*(\d+),\s*(\d+)", fn).groups())
    px = _byte_list(re.search(r"const REFERENCE: \[u8; 4\] = \[(.*?)\];", fn, re.S).group(1))
    # the compression test runs every algorithm with uniform weights (lib.rs:369-393)
    algos = re.findall(r"test\(Algorithm::([A-Za-z]+)\);", src)
    return sizes, {"format": "BC1", "width": w, "height": h, "encoded": enc, "pixel": px}, algos


def _lut_digests(lut_src):
    out = {}
    src = _strip_comments(lut_src)
    for name in ("LOOKUP_5_3", "LOOKUP_6_3", "LOOKUP_5_4", "LOOKUP_6_4"):
        start = src.index("pub const %s" % name)
        body = src[start:src.index("];", start)]
        rows = re.findall(r"entry!\(([^)]*)\)", body)
        assert len(rows) == 256, name
        blob = bytes(v for r in rows for v in _byte_list(r))
        assert len(blob) == 256 * 6
        out[name] = hashlib.sha256(blob).hexdigest()
    return out


def main(ref_root):
    here = os.path.dirname(os.path.abspath(__file__))
    rd = lambda p: open(os.path.join(ref_root, p)).read()
    data = _Eval(rd("lib/src/test_data.rs")).datasets()
    sizes, odd, algos = _lib_cases(rd("lib/src/lib.rs"))
    kat = {
        "source": "lib/src/test_data.rs:15-135, lib/src/lib.rs:350-361,369-393,416-444",
        "compression_params": {"weights": [1.0, 1.0, 1.0], "weigh_colour_by_alpha": False,
                               "algorithms": algos},
        "datasets": {k: dict(v, format=k.split("_")[0]) for k, v in data.items()},
        "storage_requirements": sizes,
        "odd_height_decode": odd,
    }
    for k, v in kat["datasets"].items():
        assert len(v["decoded"]) == 64, k
    text = json.dumps(kat, indent=1)
    # keep each byte array on one line
    text = re.sub(r"\[\s*([0-9,\s]+?)\s*\]", lambda m: "[" + ",".join(m.group(1).split()).replace(",,", ",") + "]", text)
    with open(os.path.join(here, "kat.json"), "w") as f:
        f.write(text + "\n")
    with open(os.path.join(here, "single_lut_sha256.json"), "w") as f:
        json.dump({"source": "lib/src/colourfit/single_lut.rs:52-1086",
                   "layout": "256 rows x (start0,end0,err0,start1,end1,err1) u8",
                   "sha256": _lut_digests(rd("lib/src/colourfit/single_lut.rs"))}, f, indent=1)
    print("wrote", len(data), "datasets,", len(sizes), "size cases")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: make_golden.py <path of the reference checkout>")
    main(sys.argv[1])
