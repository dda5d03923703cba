// Compile-only check that the adapters of include/flg_accel.hpp bind to the
// reference's own types: fledge::Ray (common/ray.h), SInteraction and
// VInteraction (interaction.hpp), Sampler (common/sampler.h) and Vector3f.
// Built with -fsyntax-only against the reference sources and the stand-in
// headers of oracle/refshim, where the reference is present.
#include "common/ray.h"
#include "common/sampler.h"
#include "interaction.hpp"
#include "flg_accel.hpp"

template class flg::GpuLBVH<fledge::Ray, fledge::SInteraction>;

fledge::Vector3f volume_calls(flg::DenseGridVolume &vol, const fledge::Ray &ray, fledge::Sampler &rng,
                              fledge::VInteraction &vi, bool &ok) {
  fledge::Vector3f t = vol.tr(ray, rng);
  fledge::Vector3f w = vol.sample(ray, rng, vi, ok);
  float T[1];
  vol.tr(&ray, 1, 7, T);
  return t * w;
}

bool accel_calls(flg::GpuLBVH<fledge::Ray, fledge::SInteraction> &accel, const fledge::Ray &ray,
                 fledge::SInteraction &isect) {
  return accel.intersect(ray, isect);
}
