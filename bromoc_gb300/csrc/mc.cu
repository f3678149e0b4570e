// Metropolis moves (metropolis.f90:31-55 with move.f90:19-45), device
// resident: per move a one-thread proposal, INTERACT (gcmc.cu) of the ion
// at its old position (with alerts) and at the new one, and a one-thread
// acceptance that moves the ion.  No host round trip between moves; the
// uniforms are the Philox stream mc_uniform keyed by (seed, cycle, move,
// draw), drawn in the reference's order.
#include "../../include/bromoc_gpu.h"
#include "launch.h"

namespace bgpu {

// move.f90:19-45: a mobile ion and a displacement of up to mcmax/2 per
// axis, drawn again while the new position lies outside the system (at
// most kMcTries draws; then the move is skipped).
constexpr int kMcTries = 1000;

__global__ void k_mc_propose(KP p, uint64_t seed, uint64_t cycle, int m, double mcmax,
                             McState *mc) {
  if (threadIdx.x != 0) return;
  const int ntot = p.st->ntot;
  const double natom2 = (double)(ntot - p.nsites);
  uint32_t draw = 0;
  int iat = 0;
  double xn = 0.0, yn = 0.0, zn = 0.0;
  bool found = false;
  for (int t = 0; t < kMcTries && !found; ++t) {
    iat = p.nsites + p.nfix + (int)(natom2 * mc_uniform(seed, cycle, m, draw++));  // 0-based
    xn = p.x[iat] + mcmax * (mc_uniform(seed, cycle, m, draw++) - 0.5);
    yn = p.y[iat] + mcmax * (mc_uniform(seed, cycle, m, draw++) - 0.5);
    zn = p.z[iat] + mcmax * (mc_uniform(seed, cycle, m, draw++) - 0.5);
    bool out;
    if (p.shape == 1) {
      const double r2 = (xn - p.cx) * (xn - p.cx) + (yn - p.cy) * (yn - p.cy) +
                        (zn - p.cz) * (zn - p.cz);
      out = r2 > p.rsphe2;
    } else if (p.shape == 2) {
      const double ex = (xn - p.cx) * p.iecx, ey = (yn - p.cy) * p.iecy;
      out = ex * ex + ey * ey > 1.0 || zn < p.lz2m || zn > p.lz2p;
    } else {
      out = xn < p.lx2m || xn > p.lx2p || yn < p.ly2m || yn > p.ly2p || zn < p.lz2m ||
            zn > p.lz2p;
    }
    found = !out;
  }
  mc->skip = found ? 0 : 1;
  mc->iat = iat;
  mc->draw = (int)draw;
  mc->xn = xn;
  mc->yn = yn;
  mc->zn = zn;
  Trial t{};
  t.valid = found ? 1 : 0;
  t.itype = abs(p.typei[iat]);
  t.j = iat + 1;
  t.x = p.x[iat];
  t.y = p.y[iat];
  t.z = p.z[iat];
  t.ntot = ntot;
  t.chg = -1;
  *p.trial = t;
}

// The trial at the proposed position (same ion, same slot).
__global__ void k_mc_newpos(KP p, const McState *mc) {
  if (threadIdx.x != 0) return;
  Trial t = *p.trial;
  t.x = mc->xn;
  t.y = mc->yn;
  t.z = mc->zn;
  t.e_single = 0.0;
  *p.trial = t;
}

// metropolis.f90:37-53: downhill moves are taken, uphill ones when a
// uniform falls below exp(-(enew - eold)/kT).
__global__ void k_mc_accept(KP p, uint64_t seed, uint64_t cycle, int m, McState *mc) {
  if (threadIdx.x != 0 || mc->skip) return;
  const double eold = mc->e[0], enew = mc->e[1];
  bool acc = enew <= eold;
  if (!acc) acc = mc_uniform(seed, cycle, m, (uint32_t)mc->draw) < exp(-(enew - eold) * p.ikbt);
  if (acc) {
    const int i = mc->iat;
    p.x[i] = mc->xn;
    p.y[i] = mc->yn;
    p.z[i] = mc->zn;
    mc->dener += enew - eold;
    mc->naccept += 1;
  }
}

int launch_metropolis(const KP &p, int ntot, uint32_t mask, int nmcm, double mcmax,
                      uint64_t seed, uint64_t cycle, McState *mc, cudaStream_t stream) {
  const int per_interact = 3 + (((mask & 16u) && p.qrfpar && ntot > p.nsites) ? 1 : 0);
  for (int m = 0; m < nmcm; ++m) {
    k_mc_propose<<<1, 32, 0, stream>>>(p, seed, cycle, m, mcmax, mc);
    launch_interact(p, ntot, mask, 1, &mc->e[0], stream);
    k_mc_newpos<<<1, 32, 0, stream>>>(p, mc);
    launch_interact(p, ntot, mask, 0, &mc->e[1], stream);
    k_mc_accept<<<1, 32, 0, stream>>>(p, seed, cycle, m, mc);
  }
  return nmcm * (3 + 2 * per_interact);
}

}  // namespace bgpu
