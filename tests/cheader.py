"""Prototypes of include/helmgpu.h for the static binding checks: name ->
(return type, [parameter types]), types normalised as in "const double*"."""
from __future__ import annotations

import re
from pathlib import Path

HEADER = Path(__file__).resolve().parent.parent / "include" / "helmgpu.h"


def _norm(t: str) -> str:
    return " ".join(t.replace("*", " * ").split()).replace(" *", "*")


def prototypes(text: str | None = None) -> dict[str, tuple[str, list[str]]]:
    text = HEADER.read_text() if text is None else text
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    text = "\n".join(ln for ln in text.splitlines() if not ln.lstrip().startswith("#"))
    protos = {}
    for m in re.finditer(r"([A-Za-z_][\w\s\*]*?)\b(hz_\w+)\s*\(([^;{]*?)\)\s*;", text, re.S):
        params = " ".join(m.group(3).split())
        types = []
        for p in ([] if params in ("", "void") else params.split(",")):
            p = _norm(p)
            types.append(p if p.endswith("*") else p.rsplit(" ", 1)[0])
        protos[m.group(2)] = (_norm(m.group(1)), types)
    return protos
