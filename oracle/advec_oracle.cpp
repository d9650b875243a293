/* Oracle "port" of the scalar advection app: the restated kernels
 * (advec_port.h) under the advection driver (advec_driver.h), N = 1..6 —
 * TEST INFRASTRUCTURE ONLY (see dg_oracle.h).  Linked into liboracle.so beside
 * dg_oracle.cpp, whose port::g holds the operators the kernels read. */
#include "advec_driver.h"
#include "advec_port.h"

namespace port {
template <int N>
struct AdvPolicy : A<N> {
  static void bind(void *c) { g = *(Ctx *)c; }
  static void free_ctx(void *c) { delete (Ctx *)c; }
};
}  // namespace port

static void *adv_make(const orc_ops *ops, const orc_mesh *mesh, double vel_x, double vel_y) {
  if (!ops || !mesh) { orc::g_err = "null argument"; return nullptr; }
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
  c->velX = vel_x;
  c->velY = vel_y;
  switch (N) {
    case 1: return new orc::AdvInstance<port::AdvPolicy<1>>(mesh, c);
    case 2: return new orc::AdvInstance<port::AdvPolicy<2>>(mesh, c);
    case 3: return new orc::AdvInstance<port::AdvPolicy<3>>(mesh, c);
    case 4: return new orc::AdvInstance<port::AdvPolicy<4>>(mesh, c);
    case 5: return new orc::AdvInstance<port::AdvPolicy<5>>(mesh, c);
    default: return new orc::AdvInstance<port::AdvPolicy<6>>(mesh, c);
  }
}

ADV_DEFINE_C_API
