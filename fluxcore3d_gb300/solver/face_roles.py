"""Role of each domain face (inlet / outlet / wall / periodic).

Same decision table as the reference's pre_post/face_roles.py:3-53:
the face upstream of flow_dir is the inlet, the downstream face the outlet,
`domain_walls` override everything except the inlet, `domain_outlets` add
outlets, and the remaining faces are walls when the legacy
`transverse_walls` flag is set, periodic otherwise.
"""
from __future__ import annotations

import warnings

FACES = ("+X", "-X", "+Y", "-Y", "+Z", "-Z")
AXIS = {"X": 0, "Y": 1, "Z": 2}


def flow_axis_sign(cfg) -> tuple[int, int]:
    d = cfg.flow_dir.upper().strip()
    return AXIS[d[1]], (+1 if d[0] == "+" else -1)


def resolve_face_roles(cfg) -> dict:
    axis, sign = flow_axis_sign(cfg)
    letter = "XYZ"[axis]
    inlet = ("-" if sign > 0 else "+") + letter
    outlet = ("+" if sign > 0 else "-") + letter
    walls = {s.upper().strip() for s in getattr(cfg, "domain_walls", [])}
    outlets = {s.upper().strip() for s in getattr(cfg, "domain_outlets", [])}
    legacy = bool(getattr(cfg, "transverse_walls", False))
    roles = {}
    for face in FACES:  # insertion order is the order the plane BCs are applied in
        if face == inlet:
            roles[face] = "inlet"
        elif face in walls:
            roles[face] = "wall"
        elif face == outlet or face in outlets:
            roles[face] = "outlet"
        else:
            roles[face] = "wall" if legacy else "periodic"
    if inlet in walls:
        warnings.warn(f"resolve_face_roles: '{inlet}' is the inlet face and cannot be walled; override ignored.")
    if inlet in outlets:
        warnings.warn(f"resolve_face_roles: '{inlet}' is the inlet face and cannot be an outlet; override ignored.")
    return roles


def _face_ax_idx_fsign(cfg_or_sim, face: str):
    """(axis, plane index, outward sign) of a face."""
    ax = AXIS[face[1]]
    n = (cfg_or_sim.nx, cfg_or_sim.ny, cfg_or_sim.nz)[ax]
    return (ax, n - 1, +1) if face[0] == "+" else (ax, 0, -1)


def periodic_flags(cfg) -> tuple[bool, bool, bool]:
    """Streaming periodicity: an axis is periodic unless one of its faces is inlet/outlet/wall."""
    non_periodic = {AXIS[f[1]] for f, r in resolve_face_roles(cfg).items() if r in ("inlet", "outlet", "wall")}
    return tuple(d not in non_periodic for d in range(3))
