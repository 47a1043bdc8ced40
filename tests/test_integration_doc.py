"""The Julia binding shown in INTEGRATION.md passes every C entry point as
many arguments as include/tnfa.h declares (a static check: Julia is not
installed here, so the binding itself cannot run)."""
import re
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent


def _prototypes() -> dict:
    hdr = (ROOT / "include" / "tnfa.h").read_text()
    out = {}
    for m in re.finditer(r"(?:int|const char\*|void)\s+(tnfa_\w+)\s*\(([^;]*?)\)\s*;", hdr, re.S):
        args = m.group(2).strip()
        out[m.group(1)] = 0 if args in ("", "void") else len([a for a in args.split(",") if a.strip()])
    return out


def _top_level_items(s: str) -> list:
    parts, depth, cur = [], 0, ""
    for c in s:
        depth += c in "({["
        depth -= c in ")}]"
        if c == "," and depth == 0:
            parts.append(cur)
            cur = ""
        else:
            cur += c
    parts.append(cur)
    return [p for p in parts if p.strip()]


def test_julia_ccalls_match_the_header():
    protos = _prototypes()
    doc = (ROOT / "INTEGRATION.md").read_text()
    calls = []
    for m in re.finditer(r"ccall\(\(:(tnfa_\w+),\s*lib\),\s*\w+,\s*\(", doc):
        i = j = m.end() - 1
        depth = 0
        while True:
            depth += doc[j] == "("
            depth -= doc[j] == ")"
            if depth == 0:
                break
            j += 1
        ntypes = len(_top_level_items(doc[i + 1:j]))
        # the argument values: from after the type tuple to the ccall's closing parenthesis
        k, depth = j + 1, 1
        while depth:
            depth += doc[k] == "("
            depth -= doc[k] == ")"
            k += 1
        nvals = len(_top_level_items(doc[j + 1:k - 1]))
        calls.append((m.group(1), ntypes, nvals))
    assert len(calls) >= 25
    bad = [c for c in calls if not (protos.get(c[0]) == c[1] == c[2])]
    assert not bad, bad
