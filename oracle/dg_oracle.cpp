/* Oracle "port" library: the restated kernels (port_kernels.h) driven by the
 * shared oracle driver (driver.h), for N = 1..6 — TEST INFRASTRUCTURE ONLY
 * (see dg_oracle.h). */
#include "driver.h"
#include "port_kernels.h"

namespace port {
Ctx g;

template <int N>
struct Policy : K<N> {
  static void bind(void *c) { g = *(Ctx *)c; }
  static void free_ctx(void *c) { delete (Ctx *)c; }
};
}  // namespace port

static void *orc_make(const orc_ops *ops, const orc_phys *phys, const orc_mesh *mesh, int app) {
  if (!ops || !phys || !mesh) { orc::g_err = "null argument"; return nullptr; }
  const int N = ops->N;
  if (N < 1 || N > 6) { orc::g_err = "order N must be in 1..6"; return nullptr; }
  const int Np = (N + 1) * (N + 2) / 2, Nfp = N + 1;
  auto *c = new port::Ctx();
  c->N = N;
  c->r.assign(ops->r, ops->r + Np);
  c->s.assign(ops->s, ops->s + Np);
  c->Dr.assign(ops->Dr, ops->Dr + Np * Np);
  c->Ds.assign(ops->Ds, ops->Ds + Np * Np);
  c->Drw.assign(ops->Drw, ops->Drw + Np * Np);
  c->Dsw.assign(ops->Dsw, ops->Dsw + Np * Np);
  c->LIFT.assign(ops->LIFT, ops->LIFT + Np * 3 * Nfp);
  c->FMASK.assign(ops->FMASK, ops->FMASK + 3 * Nfp);
  c->ones.assign(Np, 1.0);
  c->gam = phys->gam; c->bc_mach = phys->bc_mach; c->bc_alpha = phys->bc_alpha;
  c->bc_p = phys->bc_p; c->bc_r = phys->bc_r; c->bc_u = phys->bc_u; c->bc_v = phys->bc_v;
  c->bc_e = phys->bc_e; c->vortex_x0 = phys->vortex_x0; c->vortex_y0 = phys->vortex_y0;
  c->vortex_beta = phys->vortex_beta;
  switch (N) {
    case 1: return new orc::Instance<port::Policy<1>>(mesh, app, c);
    case 2: return new orc::Instance<port::Policy<2>>(mesh, app, c);
    case 3: return new orc::Instance<port::Policy<3>>(mesh, app, c);
    case 4: return new orc::Instance<port::Policy<4>>(mesh, app, c);
    case 5: return new orc::Instance<port::Policy<5>>(mesh, app, c);
    default: return new orc::Instance<port::Policy<6>>(mesh, app, c);
  }
}

ORC_DEFINE_C_API("port")
