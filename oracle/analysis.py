"""ORACLE -- test infrastructure only.  numpy restatement of the per-cycle
analysis of cg-gcmc-bd/src/simul1.f90:176-188 (bins) and :476-509 (rho(z)
of the mobile ions, rho(z) of the DNA sites, the RDF of the mobile ions
around particle igr), for checking the device counts."""
from __future__ import annotations

import numpy as np


def profile_bins(lz: float, cz: float, npoints: int):
    """(zmini, idelz, nzmax) as simul1.f90:179-188."""
    zmini = cz - 0.5 * lz
    idelz = 2.0
    return zmini, idelz, min(int(lz * idelz), npoints)


def accumulate(acc, x, y, z, typei, nsites, nfix, nold, typtyp, *, lz, cz, npoints,
               rho=True, rdna=False, gr=False, igr=1, dr=0.1):
    """Add one cycle's sample to acc (dict of count arrays, created on first
    use); particle arrays are 0-based, igr 1-based as in the reference."""
    zmini, idelz, nzmax = profile_bins(lz, cz, npoints)
    n = len(x)
    ntyp = int(np.abs(typei[nsites:]).max()) - nold if n > nsites else 0
    acc.setdefault("rho", np.zeros((max(ntyp, 1), nzmax)))
    acc.setdefault("rdna", np.zeros((max(int(np.max(typtyp)) if nsites else 1, 1), nzmax)))
    acc.setdefault("gr", np.zeros((max(ntyp, 1), npoints)))
    acc.setdefault("irmax", 0)
    for i in range(n):
        # iz = int((z(iat)-zmini)*idelz) + 1, int() truncating toward zero
        iz = int((z[i] - zmini) * idelz) + 1
        if i >= nsites + nfix:
            t = abs(int(typei[i])) - nold
            if rho and 1 <= iz <= nzmax:
                if t > acc["rho"].shape[0]:
                    acc["rho"] = np.pad(acc["rho"], ((0, t - acc["rho"].shape[0]), (0, 0)))
                acc["rho"][t - 1, iz - 1] += 1.0
            if gr and igr - 1 < n:
                c = igr - 1
                d = np.sqrt((x[i] - x[c]) ** 2 + (y[i] - y[c]) ** 2 + (z[i] - z[c]) ** 2)
                ir = int(d / dr) + 1
                acc["irmax"] = min(max(acc["irmax"], ir), npoints)
                if ir <= npoints:
                    if t > acc["gr"].shape[0]:
                        acc["gr"] = np.pad(acc["gr"], ((0, t - acc["gr"].shape[0]), (0, 0)))
                    acc["gr"][t - 1, ir - 1] += 1.0
        elif i < nsites and rdna and 1 <= iz <= nzmax:
            acc["rdna"][int(typtyp[i]) - 1, iz - 1] += 1.0
    return acc
