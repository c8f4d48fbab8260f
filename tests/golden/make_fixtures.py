"""Writes the golden fixtures of the test suite from the reference sources. Run it with the
environment variable REFERENCE_ROOT set to a checkout of the reference tree; the fixtures are
committed, so the tests never read the reference.

* albedo_sha256.json: sha256 of the reference's three albedo tables
  (crates/verion-gpu/tables/*.f32), which the in-tree generator must reproduce byte for byte.
"""
from __future__ import annotations

import hashlib
import json
import os
from pathlib import Path

HERE = Path(__file__).resolve().parent


def main() -> None:
    root = os.environ.get("REFERENCE_ROOT")
    if not root:
        raise SystemExit("set REFERENCE_ROOT to the reference checkout")
    tables = Path(root) / "crates" / "verion-gpu" / "tables"
    sums = {}
    for name in ("ggx_albedo.f32", "sheen_albedo.f32", "dielectric_albedo.f32"):
        data = (tables / name).read_bytes()
        sums[name] = {"sha256": hashlib.sha256(data).hexdigest(), "bytes": len(data)}
    (HERE / "albedo_sha256.json").write_text(json.dumps(sums, indent=1) + "\n")


if __name__ == "__main__":
    main()
