"""Snapshots of the gas particles: the reference's PartType0 output fields
(hydro/Minimal/hydro_io.h:180-240: Coordinates, Velocities, Masses,
SmoothingLengths, InternalEnergies, ParticleIDs, Densities, Entropies,
Pressures) and a header (BoxSize, Time, NumPart_ThisFile), plus, for a
restart, the integrator state that the output fields do not hold (full-step
velocities and energies, time bins, accelerations and rates, the integer
time line).

HDF5 is not available to this library, so the container is a NumPy ``.npz``
archive whose member names are the HDF5 paths of the reference's snapshots
("PartType0/Coordinates", "Header/BoxSize", ...).  Reading accepts the input
field names of the reference's initial conditions as well
(hydro_io.h:50-75: SmoothingLength, InternalEnergy, Density)."""
from __future__ import annotations

import numpy as np

GAMMA = np.float32(5.0 / 3.0)

# output name -> key of a box / integrator state
OUTPUT_FIELDS = {
    "Coordinates": "x", "Velocities": "v", "Masses": "m", "SmoothingLengths": "h",
    "InternalEnergies": "u", "ParticleIDs": "ids", "Densities": "rho", "Pressures": "P",
}
INPUT_ALIASES = {"SmoothingLength": "h", "InternalEnergy": "u", "Density": "rho"}
RESTART_FIELDS = ("v_full", "u_full", "a", "u_dt", "h_dt", "c", "v_sig", "time_bin",
                  "min_ngb_bin", "f", "balsara")


def entropies(u, rho):
    """gas_entropy_from_internal_energy (equation_of_state.h, ideal gas):
    (gamma - 1) u rho^-(gamma - 1), in FP32."""
    u = np.asarray(u, np.float32)
    rho = np.asarray(rho, np.float32)
    with np.errstate(divide="ignore", invalid="ignore"):
        return ((GAMMA - np.float32(1)) * u *
                np.power(rho, -(GAMMA - np.float32(1)), dtype=np.float32)).astype(np.float32)


def write(path, fields, box_size, time=0.0, restart=None):
    """Write ``fields`` (a dict with at least x, v, m, h, u; optionally ids,
    rho, P) as PartType0; ``restart`` is an optional dict of further arrays
    and scalars stored under Restart/."""
    n = int(np.asarray(fields["x"]).shape[0])
    out = {"Header/BoxSize": np.asarray(box_size, np.float64).reshape(-1),
           "Header/Time": np.float64(time),
           "Header/NumPart_ThisFile": np.array([n, 0, 0, 0, 0, 0, 0], np.int64)}
    for name, key in OUTPUT_FIELDS.items():
        if key in fields:
            out["PartType0/" + name] = np.asarray(fields[key])
    if "ids" not in fields:
        out["PartType0/ParticleIDs"] = np.arange(1, n + 1, dtype=np.uint64)
    if "rho" in fields:
        out["PartType0/Entropies"] = entropies(fields["u"], fields["rho"])
    for k, v in (restart or {}).items():
        out["Restart/" + k] = np.asarray(v)
    with open(path, "wb") as fh:
        np.savez(fh, **out)


def read(path):
    """A snapshot (or initial conditions written the same way) as a box dict:
    x, v, m, h, u, ids (and rho, P where present), dim, time, and
    ``restart`` (a dict, empty for a plain snapshot)."""
    with np.load(path, allow_pickle=False) as z:
        names = set(z.files)
        box = {}
        for name in names:
            if not name.startswith("PartType0/"):
                continue
            field = name.split("/", 1)[1]
            key = OUTPUT_FIELDS.get(field) or INPUT_ALIASES.get(field)
            if key:
                box[key] = z[name]
        for need in ("x", "v", "m", "h", "u"):
            if need not in box:
                raise KeyError(f"snapshot {path} has no PartType0 field for {need}")
        dim = z["Header/BoxSize"]
        box["dim"] = tuple(float(d) for d in (dim if dim.size == 3 else np.repeat(dim, 3)))
        box["time"] = float(z["Header/Time"]) if "Header/Time" in names else 0.0
        box["restart"] = {name.split("/", 1)[1]: z[name] for name in names
                          if name.startswith("Restart/")}
    box.setdefault("time_bin", np.zeros(box["x"].shape[0], np.int8))
    return box
