"""Regenerate ``fixture_meshes.npz`` from the reference's ASCII USD test assets.

The reference's own tests run on three bundled meshes (``examples/assets/``):
``tet_grid.usda`` (27 nodes, 40 tets), ``hex_grid.usda`` (27 nodes, 8 hexes,
VTK order) and ``tet_cantilever.usda`` (12 nodes, 10 tets).  OpenUSD (``pxr``)
is not installed, so this script reads the three plain-text attributes it needs
(``points``, ``tetVertexIndices`` and ``customData.hex_mesh.hex_vertex_indices``)
with regular expressions and stores them as arrays.  Run it where the reference
checkout is available, passing the checkout's root directory::

    python tests/golden/make_golden.py <reference checkout>
"""

import re
import sys
from pathlib import Path

import numpy as np

NUM = r"-?\d+(?:\.\d+)?(?:[eE][-+]?\d+)?"


def _tuples(text: str, name: str, width: int, dtype):
    match = re.search(rf"{re.escape(name)}\s*=\s*\[(.*?)\]", text, re.S)
    if match is None:
        return None
    values = [float(v) for v in re.findall(NUM, match.group(1))]
    return np.asarray(values, dtype=dtype).reshape(-1, width)


def parse(path: Path) -> dict:
    text = path.read_text()
    out = {"points": _tuples(text, "point3f[] points", 3, np.float64)}
    tets = _tuples(text, "int4[] tetVertexIndices", 4, np.int64)
    if tets is not None:
        out["tets"] = tets.astype(np.int32)
    hexes = _tuples(text, "int[] hex_vertex_indices", 8, np.int64)
    if hexes is not None:
        out["hexes"] = hexes.astype(np.int32)
    return out


def main(reference_root: str) -> None:
    assets = Path(reference_root) / "src/newton_solver_fem/examples/assets"
    arrays = {}
    for name in ("tet_grid", "hex_grid", "tet_cantilever"):
        for key, value in parse(assets / f"{name}.usda").items():
            arrays[f"{name}/{key}"] = value
    target = Path(__file__).with_name("fixture_meshes.npz")
    np.savez_compressed(target, **arrays)
    for key, value in arrays.items():
        print(key, value.shape, value.dtype)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py <reference checkout root>")
    main(sys.argv[1])
