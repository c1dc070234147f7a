"""Oracle for post-processing (test infrastructure): a numpy restatement of processTLBM.py's
arithmetic (python/processTLBM.py:52-186) and the XDMF skeleton of hdf5Helper.writeXdmf
(python/hdf5Helper.py:58-202).  Pinned against the script's own output in post_case.npz."""

from __future__ import annotations

import re

import numpy as np

DUMP_PLANES = ("ux", "uy", "uz", "velmag", "Fx", "Fy", "Fz", "pressure")
AVG_PLANES = ("ux", "uy", "uz", "velmag", "pressure")
H5_NAME = {"ux": "velo_group/x_velo", "uy": "velo_group/y_velo", "uz": "velo_group/z_velo",
           "velmag": "velo_group/velmag", "Fx": "force_group/x_force",
           "Fy": "force_group/y_force", "Fz": "force_group/z_force",
           "pressure": "pres_group/presmag"}


def parse_params(text: str) -> dict:
    t = text.split()
    return {"num_ts": int(t[2]), "warmup": int(t[4]), "plot_freq": int(t[5]), "nx": int(t[10]),
            "ny": int(t[11]), "nz": int(t[12]), "time_avg": int(t[14]), "lx": float(t[15]),
            "t_conv": float(t[18]), "l_conv": float(t[19]), "p_conv": float(t[20]),
            "p_ref_idx": int(t[21])}


def process(p: dict, order, ux, uy, uz, rho, fx=None, fy=None, fz=None, time_avg=False):
    """Fields in global order as processTLBM computes them (float32 inputs)."""
    u_conv = p["t_conv"] / p["l_conv"]                                  # :52
    ux, uy, uz, rho = (np.array(a, np.float32) for a in (ux, uy, uz, rho))
    if time_avg:                                                        # :150-153
        ux /= p["num_ts"]
        uy /= p["num_ts"]
        uz /= p["num_ts"]
        rho /= p["num_ts"]
    ux /= u_conv                                                        # :83-86
    uy /= u_conv
    uz /= u_conv
    rho *= p["p_conv"]
    out = {}
    for k, a in (("ux", ux), ("uy", uy), ("uz", uz), ("pressure", rho)):  # :89-94
        g = np.zeros_like(a)
        g[order] = a
        out[k] = g
    out["pressure"] -= out["pressure"][p["p_ref_idx"]]                  # :95-96
    out["velmag"] = np.sqrt(out["ux"] ** 2 + out["uy"] ** 2 + out["uz"] ** 2)  # :98
    if not time_avg:
        f_conv = p["l_conv"] / u_conv ** 2                               # :101
        for k, a in (("Fx", fx), ("Fy", fy), ("Fz", fz)):               # :107-113
            a = np.array(a, np.float32)
            a *= f_conv
            g = np.zeros_like(a)
            g[order] = a
            out[k] = g
    return out


def xdmf_skeleton(text: str) -> str:
    """The XDMF with every heavy-data reference removed: HDF items (``file.h5:/group/ds``) and
    binary items (file name, precision, endianness, byte offset) compare equal."""
    text = re.sub(r' NumberType="Float"( Precision="4")?( Format="(HDF|Binary)")'
                  r'( Endian="Little")?( Seek="\d+")?>\n[^\n<]+\n', ' NumberType="Float">\nDATA\n',
                  text)
    return text
