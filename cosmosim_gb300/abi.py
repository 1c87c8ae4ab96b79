"""numpy views of the C structs shared with cosmosim's callers.

The dtypes below have the byte layout of ``Body`` (168 B, reference
src/body.h:13-27) and ``OctreeNode`` (104 B, reference src/octree.h:6-14), so a
numpy array of them can be passed to the C entry points as ``Body*`` /
``OctreeNode*`` unchanged.
"""
import ctypes

import numpy as np

BODY_STAR, BODY_GAS, BODY_SMBH, BODY_JET, BODY_DUST, BODY_LOBE = range(6)

BODY_DTYPE = np.dtype(
    {
        "names": [
            "x", "y", "z", "vx", "vy", "vz", "ax", "ay", "az", "mass", "type",
            "spin_x", "spin_y", "spin_z", "accretion_rate", "luminosity", "lifetime",
            "density", "pressure", "internal_energy", "smoothing_h",
        ],
        "formats": ["<f8"] * 10 + ["<i4"] + ["<f8"] * 10,
        "offsets": [0, 8, 16, 24, 32, 40, 48, 56, 64, 72, 80,
                    88, 96, 104, 112, 120, 128, 136, 144, 152, 160],
        "itemsize": 168,
    }
)

NODE_DTYPE = np.dtype(
    {
        "names": ["cx", "cy", "cz", "total_mass", "center_x", "center_y", "center_z",
                  "half_size", "body_index", "children"],
        "formats": ["<f8"] * 8 + ["<i4", ("<i4", (8,))],
        "offsets": [0, 8, 16, 24, 32, 40, 48, 56, 64, 68],
        "itemsize": 104,
    }
)


class CosmosimConfig(ctypes.Structure):
    """reference src/cosmosim_api.h:16-27 (72 bytes)."""

    _fields_ = [
        ("n_bodies", ctypes.c_int),
        ("merger", ctypes.c_int),
        ("quasar", ctypes.c_int),
        ("dt", ctypes.c_double),
        ("theta", ctypes.c_double),
        ("smbh_mass_frac", ctypes.c_double),
        ("accretion_radius", ctypes.c_double),
        ("jet_speed", ctypes.c_double),
        ("feedback_strength", ctypes.c_double),
        ("substeps", ctypes.c_int),
    ]


assert ctypes.sizeof(CosmosimConfig) == 72


class QuasarConfig(ctypes.Structure):
    """reference src/quasar.h:6-22 (104 bytes)."""

    _fields_ = [(f, ctypes.c_double) for f in (
        "accretion_radius", "swallow_radius", "isco_radius", "viscosity_alpha", "jet_speed",
        "jet_mass", "jet_lifetime", "feedback_strength", "eta_eff", "eddington_k",
        "accretion_smoothing")] + [(f, ctypes.c_int) for f in (
            "jet_cap", "jet_count", "max_bodies", "jet_ring_count")]


assert ctypes.sizeof(QuasarConfig) == 104


def new_bodies(n):
    """Zeroed Body array (what calloc gives the reference's callers)."""
    return np.zeros(n, dtype=BODY_DTYPE)


def new_pool(n_nodes):
    return np.zeros(n_nodes, dtype=NODE_DTYPE)


def ptr(a):
    """Raw data pointer of a C-contiguous numpy array, as c_void_p.

    Structured arrays must have exactly the ABI layout: numpy operations such
    as concatenate repack padded dtypes (Body becomes 164 bytes), and such an
    array would be read with the wrong stride."""
    if not a.flags["C_CONTIGUOUS"]:
        raise ValueError("array must be C-contiguous")
    if a.dtype.names is not None and a.dtype not in (BODY_DTYPE, NODE_DTYPE):
        raise TypeError(f"structured array has layout {a.dtype.itemsize} B, not the Body "
                        f"({BODY_DTYPE.itemsize} B) or OctreeNode ({NODE_DTYPE.itemsize} B) ABI; "
                        "use .astype(BODY_DTYPE)")
    return ctypes.c_void_p(a.ctypes.data)
