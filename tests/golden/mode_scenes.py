"""Scenes for the field-mode comparisons: the texture_variants "default" scene
(2x2x2 blocks of depth 3-4, 10 % masked nodes, 160x120) with a secondary field
on the same nodes (linear in world coordinates), and per mode the view
threshold and presentation the reference's renderer would set
(DenseFieldRenderer_cu.cu:418-445)."""
from __future__ import annotations

import numpy as np

import texture_variants as tv
from revise_gb300 import _lib, host

MODES = {
    "isosurface": _lib.MODE_ISOSURFACE,
    "isosurfaces": _lib.MODE_ISOSURFACES,
    "max_intensity": _lib.MODE_MAX_INTENSITY,
    "argb_light": _lib.MODE_ARGB_LIGHT,
    "domain_voxels": _lib.MODE_DOMAIN_VOXELS,
    "value_on_isosurface": _lib.MODE_VALUE_ON_ISOSURFACE,
    "value_on_isosurfaces": _lib.MODE_VALUE_ON_ISOSURFACES,
}


def scene(name: str, filt: int = _lib.FILTER_TEXTURE):
    """(workload, view, presentation, secondary sparse values or None)."""
    w = tv.workload("default")
    mode = MODES[name]
    view = host.view_for(w, filter=filt)
    span = w.field_max - w.field_min
    rel = lambda r: float(np.float32(w.field_min + r * span))  # noqa: E731 (relToAbsFieldValue)
    if mode in (_lib.MODE_ISOSURFACE, _lib.MODE_VALUE_ON_ISOSURFACE):
        view.threshold = rel(0.45)
    elif mode in (_lib.MODE_ISOSURFACES, _lib.MODE_VALUE_ON_ISOSURFACES):
        view.threshold = 0.0
    levels = [rel(x) for x in (0.2, 0.35, 0.5, 0.65, 0.8)] if mode in (
        _lib.MODE_ISOSURFACES, _lib.MODE_VALUE_ON_ISOSURFACES) else []
    sparse2 = None
    srange = (0.0, 1.0)
    if mode in (_lib.MODE_VALUE_ON_ISOSURFACE, _lib.MODE_VALUE_ON_ISOSURFACES):
        sparse2 = np.empty_like(w.sparse)
        for b in range(w.nblocks):
            a, c = int(w.node_off[b]), int(w.node_off[b + 1])
            u = w.n2i[a:c].astype(np.float64) / (1 << int(w.blocks[b, 3])) + w.blocks[b, :3]
            sparse2[a:c] = (0.25 * u[:, 0] + 0.2 * u[:, 1] + 0.1 * u[:, 2]).astype(np.float32)
        srange = (0.0, 1.1)
    pres = host.presentation(mode, view, isosurface_opacity=0.6, levels=levels, secondary_range=srange)
    return w, view, pres, sparse2


def clear_value(pres) -> int:
    """clearViewport's fill: NaN bits for max-intensity, else 0 (DenseFieldRenderer_cu.cu:268-277)."""
    return 0x7FC00000 if pres.mode == _lib.MODE_MAX_INTENSITY else 0
