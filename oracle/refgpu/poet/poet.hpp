// BASELINE ONLY: a project-written stand-in for the POET dispatch header,
// which the reference's CUDA sources include (<poet/poet.hpp>) and which its
// build fetches over the network. It is used to compile the reference
// cuFINUFFT as a same-box GPU baseline (oracle/Makefile, target ref-gpu) and
// is never part of the GB300 engine. It provides the three names those
// sources use: inclusive_range<Lo, Hi>, dispatch_param<Range>{value} and
// dispatch(f, tuple_of_params, args...), which calls
// f.template operator()<V0, V1, ...>(args...) with each Vi the compile-time
// value of range i equal to the runtime value of parameter i.
#pragma once
#include <cstddef>
#include <stdexcept>
#include <tuple>
#include <type_traits>
#include <utility>

namespace poet {

template <int Lo, int Hi> struct inclusive_range {};
template <class Range> struct dispatch_param {
  int value;
};

namespace detail {
template <class P> struct range_of;
template <int Lo, int Hi> struct range_of<dispatch_param<inclusive_range<Lo, Hi>>> {
  static constexpr int lo = Lo;
  static constexpr int hi = Hi;
};

template <class Ret, class F, class Tup, std::size_t I, int... Vs> struct Disp {
  template <class... A> static Ret go(F &f, const Tup &t, A &&...a) {
    if constexpr (I == std::tuple_size_v<Tup>) {
      return f.template operator()<Vs...>(std::forward<A>(a)...);
    } else {
      using R = range_of<std::remove_cv_t<std::tuple_element_t<I, Tup>>>;
      return scan<R::lo, R::hi>(f, t, std::get<I>(t).value, std::forward<A>(a)...);
    }
  }
  template <int V, int Hi, class... A>
  static Ret scan(F &f, const Tup &t, int want, A &&...a) {
    if (want == V) return Disp<Ret, F, Tup, I + 1, Vs..., V>::go(f, t, std::forward<A>(a)...);
    if constexpr (V < Hi) return scan<V + 1, Hi>(f, t, want, std::forward<A>(a)...);
    else throw std::invalid_argument("dispatch value outside its range");
  }
};

template <class F, class Tup, std::size_t... Is, class... A>
auto first_result(F &f, std::index_sequence<Is...>, A &&...a)
    -> decltype(f.template operator()<range_of<std::remove_cv_t<std::tuple_element_t<Is, Tup>>>::lo...>(
        std::forward<A>(a)...));
} // namespace detail

template <class F, class Tup, class... A> decltype(auto) dispatch(F &&f, const Tup &t, A &&...a) {
  using FF = std::remove_reference_t<F>;
  using Ret = decltype(detail::first_result<FF, Tup>(
      std::declval<FF &>(), std::make_index_sequence<std::tuple_size_v<Tup>>{},
      std::declval<A>()...));
  FF &fr = f;
  return detail::Disp<Ret, FF, Tup, 0>::go(fr, t, std::forward<A>(a)...);
}

} // namespace poet
