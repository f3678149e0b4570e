"""The oracle's MMIJ reaction field on the CPU.  RECTBOX (rect_rf1/rf0): the
forces are the gradient of the energy (central differences), and INTERACT
of an ion is E(all) - E(all without it) for present ions and insertion
trials.  SPHERE (sphe_rf0): INTERACT against the multipole basis formed
independently from scipy's associated Legendre functions."""
import math

import numpy as np
import pytest

from bromoc_gb300 import abi

from . import systems


def _energy(o, mask=abi.M_MMIJ):
    return o.energy(mask, forces=False)[0]["ener"]


def test_rect_forces_are_gradients(oracle_mod):
    spec = systems.mmij("rect")
    o = oracle_mod.create(4000)
    spec.push(o)
    t, f, _ = o.energy(abi.M_MMIJ, forces=True)
    assert t["egsbpb"] != 0.0 and t["ener"] == t["egsbpb"]
    x, y, z, ty = spec.x.copy(), spec.y.copy(), spec.z.copy(), spec.typei.copy()
    inside = [i for i in range(len(x)) if abs(x[i]) < 8.9 and abs(y[i]) < 8.9 and
              abs(z[i]) < 11.9][:10]
    assert len(inside) >= 5
    h = 1e-5
    for i in inside:
        for a, arr in enumerate((x, y, z)):
            v = arr[i]
            e = []
            for d in (-h, h):
                arr[i] = v + d
                o.set_particles(x, y, z, ty, spec.nsites, spec.nfix)
                e.append(_energy(o))
            arr[i] = v
            fd = -(e[1] - e[0]) / (2 * h)
            assert abs(fd - f[i, a]) <= 1e-6 * max(1.0, np.abs(f).max()), (i, a, fd, f[i, a])


@pytest.mark.parametrize("shape", ["rect", "sphere"])
def test_interact_is_the_energy_difference(oracle_mod, shape):
    """rf0 = E(coef) - E(coef without j) on the same basis as rf1 (RECTBOX;
    for SPHERE the rf0 basis is the 1/sin(theta) one, so only RECTBOX
    compares with ENERGY: SPHERE checks removal by two rf0 calls)."""
    spec = systems.mmij(shape)
    o = oracle_mod.create(4000)
    spec.push(o)
    n = len(spec.x)
    e_all = _energy(o)
    x, y, z, ty = spec.x, spec.y, spec.z, spec.typei
    for j in (3, 17, 40, n - 1):
        de = o.interact(x[j], y[j], z[j], abs(int(ty[j])), j + 1, abi.M_MMIJ)
        if shape == "rect":
            keep = np.arange(n) != j
            o2 = oracle_mod.create(4000)
            spec.push(o2)
            o2.set_particles(x[keep], y[keep], z[keep], ty[keep], spec.nsites, spec.nfix)
            assert de == pytest.approx(e_all - _energy(o2), rel=1e-10, abs=1e-12)
        else:
            assert math.isfinite(de)
    # an insertion trial at a fresh point inside the region
    de = o.interact(1.0, -2.0, 3.0, spec.nold + 1, n + 1, abi.M_MMIJ)
    if shape == "rect":
        o3 = oracle_mod.create(4000)
        spec.push(o3)
        o3.set_particles(np.append(x, 1.0), np.append(y, -2.0), np.append(z, 3.0),
                         np.append(ty, spec.nold + 1), spec.nsites, spec.nfix)
        assert de == pytest.approx(_energy(o3) - e_all, rel=1e-10, abs=1e-12)


def test_sphere_interact_against_scipy_multipoles(oracle_mod):
    special = pytest.importorskip("scipy.special")
    spec = systems.mmij("sphere")
    mm = spec.mmij
    nm, R = mm["nmpol"], mm["srdist"]
    M = np.triu(mm["mmij"]) + np.triu(mm["mmij"], 1).T
    # basis order of sphe_svpol and the norms of sphe_norm
    lm = []
    for l in range(nm):
        lm.append((l, 0))
        for m in range(1, l + 1):
            lm += [(l, m), (l, -m)]
    norm = []
    for l, m in lm:
        lp = (2 * l + 1) * (2 * l + 3) / (4 * math.pi if m == 0 else 2 * math.pi)
        if l == 0:
            lp = 1.5 / (2 * math.pi)
        norm.append(math.sqrt(lp * math.factorial(l - abs(m)) /
                              (R ** (2 * l + 3) * math.factorial(l + abs(m)))))
    norm = np.array(norm)

    def basis(p):
        r = np.linalg.norm(p)
        ct, phi = p[2] / r, math.atan2(p[1], p[0])
        out = []
        for (l, m), nrm in zip(lm, norm):
            P = (-1) ** abs(m) * special.lpmv(abs(m), l, ct)  # no Condon-Shortley phase
            ang = 1.0 if m == 0 else (math.cos(m * phi) if m > 0 else math.sin(-m * phi))
            out.append(nrm * r ** l * P * ang)
        return np.array(out)

    o = oracle_mod.create(4000)
    spec.push(o)
    pos = np.stack([spec.x, spec.y, spec.z], 1)
    q = np.array([spec.ion_cg[abs(int(t)) - spec.nold - 1] for t in spec.typei])
    inside = [i for i in range(len(pos)) if np.dot(pos[i], pos[i]) <= R * R]
    coef = sum(q[i] * basis(pos[i]) for i in inside)
    e = lambda c: 0.5 * c @ M @ c
    j = inside[len(inside) // 2]
    de = o.interact(*pos[j], abs(int(spec.typei[j])), j + 1, abi.M_MMIJ)
    ref = e(coef) - e(coef - q[j] * basis(pos[j]))
    # the oracle multiplies by celec: compare the ratio against the constant
    ratio = de / ref
    assert ratio == pytest.approx(332.0637, rel=1e-4), ratio
    j2 = inside[0]
    de2 = o.interact(*pos[j2], abs(int(spec.typei[j2])), j2 + 1, abi.M_MMIJ)
    ref2 = e(coef) - e(coef - q[j2] * basis(pos[j2]))
    assert de2 / ref2 == pytest.approx(ratio, rel=1e-9)
