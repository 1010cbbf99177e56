"""Cubiquity's volume metadata (.toml beside a .dag): material names and colours.

The layout follows the reference's Metadata::load / save
(src/application/base/metadata.cpp:33-107): an optional
`dimensions = [x, y, z]`, then an array of tables `[[materials]]`, one per
material index, each with an optional `name` and an optional
`base_color = [r, g, b]` written with four decimals.  Missing colours default
to 0.8 grey (metadata.h DefaultColor).
"""
from __future__ import annotations

import tomllib
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

DEFAULT_COLOR = (0.8, 0.8, 0.8)


@dataclass
class Material:
    name: str | None = None
    base_color: tuple | None = None

    def color(self) -> tuple:
        return self.base_color if self.base_color is not None else DEFAULT_COLOR


@dataclass
class Metadata:
    dimensions: tuple | None = None
    materials: list = field(default_factory=list)
    header: str = ""


def load(path) -> Metadata:
    with open(path, "rb") as f:
        data = tomllib.load(f)
    dims = data.get("dimensions")
    meta = Metadata(dimensions=tuple(int(v) for v in dims) if dims is not None else None)
    for entry in data.get("materials", []):
        col = entry.get("base_color")
        meta.materials.append(Material(entry.get("name"), tuple(float(v) for v in col) if col is not None else None))
    return meta


def dumps(meta: Metadata) -> str:
    out = []
    if meta.header:
        out.append(meta.header + "\n")
    if meta.dimensions is not None:
        out.append("# Dimensions\n# ----------\n# These are dimensions of the volume (and array) along the x, y and z "
                   "axis.\n\n")
        out.append("dimensions = [{}, {}, {}]\n\n".format(*meta.dimensions))
    if meta.materials:
        out.append("# Materials\n# ---------\n# One table per material index (8-bit voxels: up to 256).\n\n")
    for i, m in enumerate(meta.materials):
        out.append(f"[[materials]] # Material index {i}\n")
        if m.name is not None:
            out.append('name = "{}"\n'.format(m.name.replace("\\", "\\\\").replace('"', '\\"')))
        if m.base_color is not None:
            out.append("base_color = [{:.4f}, {:.4f}, {:.4f}]\n".format(*m.base_color))
        out.append("\n")
    return "".join(out)


def save(path, meta: Metadata) -> None:
    Path(path).write_text(dumps(meta))


def material_table(meta: Metadata, emission: dict | None = None) -> np.ndarray:
    """(256, 2, 3) albedo/emission table for the pathtracer: albedo = each
    material's base colour (default grey), emission from `emission`
    {index: (r, g, b)}."""
    t = np.zeros((256, 2, 3), np.float32)
    t[:, 0] = DEFAULT_COLOR
    for i, m in enumerate(meta.materials[:256]):
        t[i, 0] = m.color()
    for i, e in (emission or {}).items():
        t[i, 1] = e
    return t
