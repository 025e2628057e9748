// pn_traverse_sph.cuh -- foreach_point_neighbor for the WCSPH (density, force, step) and
// adjoint pair functions, instantiated in pn_traverse_{f32,f64,mixed}_sph.cu.
#pragma once

#include "pn_traverse_impl.cuh"

namespace pn {

template <typename T, typename V>
int foreach_sph(pn_search* s, int32_t functor, int64_t n_x, const void* params,
                TravCall<T>& c, cudaStream_t st) {
  constexpr bool kMixed = !std::is_same<T, V>::value;
  TravArgs<T>& a = c.a;
  MixedGeom& m = c.m;
  const bool sorted = c.sorted, cache_on = c.cache_on;
  const int64_t n_sorted = c.n_sorted, n_launch = c.n_launch;
  auto use_cache = [&]() {
    if (c.fast) use_pair_cache(s, c.a32);  // a mixed search's Float32 traversal
    else use_pair_cache(s, a);
  };
  switch (functor) {
    case PN_F_WCSPH_DENSITY:
    case PN_F_WCSPH_STEP: {
      const auto* u = static_cast<const pn_wcsph_params*>(params);
      const bool step = functor == PN_F_WCSPH_STEP;
      if (step && !sorted) return PN_ERR_INVALID_ARG;
      DensityParams<V> p{sph_const<V>(s, u), static_cast<V*>(u->density),
                         static_cast<V*>(u->pressure), static_cast<const V*>(u->velocity),
                         nullptr, nullptr};
      if (sorted && u->velocity != nullptr) {
        p.pa = static_cast<V*>(s->d_pa);
        p.pb = static_cast<V*>(s->d_pb);
      }
      int rc = PN_OK;
      bool done = false;
      if constexpr (std::is_same<T, double>::value && !kMixed) {
        if (cache_on && !s->pc_valid && c.fast64 && df64_usable(s)) {
          // double-float sums: record the neighbours (decisions only), then sum over the
          // cache below
          MaskPairParams<NoneParams> pm{NoneParams{}, {}};
          rc = pc_prepare(s, n_sorted, &pm.m, st);
          if (rc == PN_OK) {
            const DF64Params<MaskPairParams<NoneParams>> dp{
                pm, c.g64, df64_geom(s, p.c, nullptr, (double)c.a32.g.r)};
            rc = launch_df64<DF64<3, FNoneMask<double, 3>>>(c.a32, dp, n_launch, st);
          }
          if (rc != PN_OK) return rc;
          s->pc_valid = true;
          use_cache();
        }
      }
      if (cache_on && !s->pc_valid) {
        MaskPairParams<DensityParams<V>> pp{p, {}};
        rc = pc_prepare(s, n_sorted, &pp.m, st);
        if (rc == PN_OK) {
          if constexpr (kMixed) {
            const MixedParams<MaskPairParams<DensityParams<V>>> mp{pp, m};
            rc = launch_trav<float, MixedFastOf<FDensityMask>::template type>(
                s, c.a32, mp, sorted, n_launch, st);
          } else {
            bool via32 = false;  // Float64: the Float32 traversal, each candidate in Float64
            if constexpr (std::is_same<T, double>::value) {
              if (c.fast64 && s->ndims >= 2) {
                const Exact64Params<MaskPairParams<DensityParams<V>>> ep{pp, c.g64};
                rc = launch_trav<float, Exact64Of<FDensityMask>::template type>(
                    s, c.a32, ep, sorted, n_launch, st);
                via32 = true;
              }
            }
            if (!via32) rc = launch_trav<T, FDensityMask>(s, a, pp, sorted, n_launch, st);
          }
        }
        if (rc == PN_OK) {
          s->pc_valid = true;
          use_cache();
        }
        done = true;
      }
      if (!done) rc = launch_pair<T, V, FDensity>(s, a, p, m, sorted, n_launch, st, c.fast_args(), c.fast64_args(), c.geom64());
      if (rc != PN_OK || !step) return rc;
      ForceParams<V> pf{p.c, static_cast<const V*>(s->d_pa), static_cast<const V*>(s->d_pb),
                        static_cast<V*>(u->accel)};
      use_state(s, a, m, c, pf.pa);
      return launch_pair<T, V, FForce>(s, a, pf, m, sorted, n_launch, st, c.fast_args(), c.fast64_args(), c.geom64());
    }
    case PN_F_WCSPH_FORCE: {
      const auto* u = static_cast<const pn_wcsph_params*>(params);
      if (!sorted) return PN_ERR_INVALID_ARG;
      const int b = div_up(n_sorted, 256);
      const int32_t* n_slots = s->ovf_active ? s->d_ovf_start + s->n_total : s->d_start + s->n_total;
      const T* pos = static_cast<const T*>(s->d_pos);
      V* pa = static_cast<V*>(s->d_pa);
      V* pb = static_cast<V*>(s->d_pb);
      const V* dn = static_cast<const V*>(u->density);
      const V* pr = static_cast<const V*>(u->pressure);
      const V* ve = static_cast<const V*>(u->velocity);
      if (b > 0 && !u->reuse_state) {
        const int32_t ns = (int32_t)n_sorted;
        switch (s->ndims) {
          case 1: k_gather_state<T, V, 1><<<b, 256, 0, st>>>(s->d_perm, pos, ns, n_slots, dn, pr, ve, pa, pb); count_launch(); break;
          case 2: k_gather_state<T, V, 2><<<b, 256, 0, st>>>(s->d_perm, pos, ns, n_slots, dn, pr, ve, pa, pb); count_launch(); break;
          default: k_gather_state<T, V, 3><<<b, 256, 0, st>>>(s->d_perm, pos, ns, n_slots, dn, pr, ve, pa, pb, reinterpret_cast<float4*>(s->d_sdf)); count_launch(); break;
        }
      }
      ForceParams<V> pf{sph_const<V>(s, u), pa, pb, static_cast<V*>(u->accel)};
      use_state(s, a, m, c, pf.pa);
      return launch_pair<T, V, FForce>(s, a, pf, m, sorted, n_launch, st, c.fast_args(), c.fast64_args(), c.geom64());
    }
    case PN_F_ADJOINT_FORWARD:
    case PN_F_ADJOINT_BACKWARD: {
      const auto* u = static_cast<const pn_adjoint_params*>(params);
      if (!sorted || !(u->cutoff > 0.0) || !(u->h > 0.0)) return PN_ERR_INVALID_ARG;
      pn_wcsph_params w{};
      w.mass = u->mass;
      w.h = u->h;
      w.c0 = w.rho0 = w.gamma_exp = 1.0;
      AdjointParams<V> p{};
      p.c = sph_const<V>(s, &w);
      p.cutoff = (V)u->cutoff;
      p.inv_cutoff = (V)(1.0 / u->cutoff);
      p.cutoff2 = p.cutoff * p.cutoff;
      p.lambda = (V)u->lambda_pot;
      p.pa = static_cast<V*>(s->d_pa);
      if (functor == PN_F_ADJOINT_FORWARD) {
        if (!u->density || !u->terms || !u->loss) return PN_ERR_INVALID_ARG;
        int rc = ensure_sum_part(s);
        if (rc != PN_OK) return rc;
        p.density = static_cast<V*>(u->density);
        p.terms = static_cast<V*>(u->terms);
        bool done = false;
        if (cache_on && !s->pc_valid) {
          MaskPairParams<AdjointParams<V>> pp{p, {}};
          rc = pc_prepare(s, n_sorted, &pp.m, st);
          if (rc == PN_OK) {
            if constexpr (kMixed) {
              const MixedParams<MaskPairParams<AdjointParams<V>>> mp{pp, m};
              rc = launch_trav<float, MixedFastOf<FAdjointForwardMask>::template type>(
                  s, c.a32, mp, sorted, n_launch, st);
            } else {
              bool via32 = false;
              if constexpr (std::is_same<T, double>::value) {
                if (c.fast64 && s->ndims >= 2) {
                  const Exact64Params<MaskPairParams<AdjointParams<V>>> ep{pp, c.g64};
                  rc = launch_trav<float, Exact64Of<FAdjointForwardMask>::template type>(
                      s, c.a32, ep, sorted, n_launch, st);
                  via32 = true;
                }
              }
              if (!via32) rc = launch_trav<T, FAdjointForwardMask>(s, a, pp, sorted, n_launch, st);
            }
          }
          if (rc == PN_OK) s->pc_valid = true;
          done = true;
        }
        if (!done)
          rc = launch_pair<T, V, FAdjointForward>(s, a, p, m, sorted, n_launch, st,
                                                  c.fast_args(), c.fast64_args(), c.geom64());
        if (rc != PN_OK) return rc;
        k_sum_partials<V><<<SUM_BLOCKS, 256, 0, st>>>(p.terms, n_x, s->d_sum_part); count_launch();
        k_sum_final<<<1, 256, 0, st>>>(s->d_sum_part, SUM_BLOCKS, u->loss); count_launch();
        return cuda_status(cudaGetLastError());
      }
      if (!u->grad || (!u->reuse_state && !u->density)) return PN_ERR_INVALID_ARG;
      if (!u->reuse_state) {
        const int b = div_up(n_sorted, 256);
        const int32_t* n_slots = s->ovf_active ? s->d_ovf_start + s->n_total : s->d_start + s->n_total;
        const T* pos = static_cast<const T*>(s->d_pos);
        const V* dn = static_cast<const V*>(u->density);
        const int32_t ns = (int32_t)n_sorted;
        if (b > 0) {
          switch (s->ndims) {
            case 1: k_gather_adjoint<T, V, 1><<<b, 256, 0, st>>>(s->d_perm, pos, ns, n_slots, dn, p.pa); count_launch(); break;
            case 2: k_gather_adjoint<T, V, 2><<<b, 256, 0, st>>>(s->d_perm, pos, ns, n_slots, dn, p.pa); count_launch(); break;
            default: k_gather_adjoint<T, V, 3><<<b, 256, 0, st>>>(s->d_perm, pos, ns, n_slots, dn, p.pa); count_launch(); break;
          }
        }
      }
      p.grad = static_cast<V*>(u->grad);
      p.scale = u->grad_scale;
      use_state(s, a, m, c, static_cast<const V*>(p.pa));
      return launch_pair<T, V, FAdjointBackward>(s, a, p, m, sorted, n_launch, st,
                                                 c.fast_args(), c.fast64_args(), c.geom64());
    }
    default:
      return PN_ERR_UNSUPPORTED_FUNCTOR;
  }
}

}  // namespace pn
