"""Device-resident copies of a chemistry workload (torch CUDA tensors in the
reference's Fortran layout), for the *_dev entry points. torch supplies the
device memory and streams only; all computation is in libreprobus_gb300.so."""
from __future__ import annotations

import numpy as np

FIELDS_IN = ("alt", "trajlon", "trajlat", "trajpre", "trajtem")
FIELDS_STATE = ("qj1", "hc", "vsed3d", "parth2osed", "parthno3sed", "surfarea", "sza3d")


def _flat(a):
    return np.ascontiguousarray(a.reshape(-1, order="F"))


class DeviceCase:
    """Uploads the arrays of an inputs.ChemCase (or a state dict) to the GPU."""

    def __init__(self, case, device="cuda", state=None):
        import torch
        self.case = case
        st = case.state_copy() if state is None else state
        self.t = {}
        for f in FIELDS_IN:
            self.t[f] = torch.from_numpy(_flat(getattr(case, f))).to(device)
        for f in FIELDS_STATE:
            self.t[f] = torch.from_numpy(_flat(st[f])).to(device)

    def __getitem__(self, k):
        return self.t[k]

    def args(self):
        """Positional arrays of ChemStep.step_dev after (ilat0, ilat1, daynum, dt)."""
        c, t = self.case, self.t
        return (t["alt"], t["trajlon"], t["trajlat"], t["trajpre"], t["trajtem"], c.irapp, t["qj1"], t["hc"],
                t["vsed3d"], t["parth2osed"], t["parthno3sed"], t["surfarea"], t["sza3d"])

    def state_host(self):
        """Copies the state back into Fortran-ordered numpy arrays shaped like the case's."""
        c = self.case
        out = {}
        for f in FIELDS_STATE:
            shape = getattr(c, f).shape
            out[f] = self.t[f].cpu().numpy().reshape(shape, order="F")
        return out
