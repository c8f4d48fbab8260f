"""Writes the golden fixtures of the test suite from the reference sources (run in a checkout
that has the reference tree at REFERENCE_ROOT; the fixtures are committed, so the tests never
read the reference).

* albedo_sha256.json: sha256 of the reference's three albedo tables
  (crates/verion-gpu/tables/*.f32), which the in-tree generator must reproduce byte for byte.
"""
from __future__ import annotations

import hashlib
import json
import os
from pathlib import Path

HERE = Path(__file__).resolve().parent
REFERENCE_ROOT = Path(os.environ.get("REFERENCE_ROOT", "/root/reference"))


def main() -> None:
    tables = REFERENCE_ROOT / "crates" / "verion-gpu" / "tables"
    sums = {}
    for name in ("ggx_albedo.f32", "sheen_albedo.f32", "dielectric_albedo.f32"):
        data = (tables / name).read_bytes()
        sums[name] = {"sha256": hashlib.sha256(data).hexdigest(), "bytes": len(data)}
    (HERE / "albedo_sha256.json").write_text(json.dumps(sums, indent=1) + "\n")


if __name__ == "__main__":
    main()
