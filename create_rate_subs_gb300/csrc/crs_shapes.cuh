// Reaction "shapes" for the fast kernels.
//
// One thread evaluates one state, so a reaction's dependency chain (rate
// exponent -> exp -> product -> net rate) is serial, and with the few warps
// per SM that the per-thread shared-memory columns allow, that latency is
// what bounds the kernels.  The host therefore groups reactions with the
// same stoichiometric shape -- reactant factors NR, product factors NP,
// net-nu entries NNU, reversible, exponential rate form, no pressure
// modification -- and the kernels evaluate four reactions of a group at a
// time with compile-time trip counts: four independent chains per thread.
// Reactions of any other form go through the general per-reaction path.
// Only the order in which reactions add into wdot changes.
#pragma once

namespace crs {

struct Shape {
  int nr, np, nnu, rev;
};

// The shapes with specialised code paths (2->2 reversible first: it is by
// far the most common elementary form).
constexpr int NSHAPE = 11;
__host__ __device__ constexpr Shape shape_of(int s) {
  return s == 0 ? Shape{2, 2, 4, 1}
       : s == 1 ? Shape{2, 3, 5, 1}
       : s == 2 ? Shape{2, 2, 4, 0}
       : s == 3 ? Shape{1, 2, 3, 1}
       : s == 4 ? Shape{2, 1, 3, 1}
       : s == 5 ? Shape{3, 2, 5, 1}
       : s == 6 ? Shape{2, 3, 3, 1}
       : s == 7 ? Shape{3, 2, 3, 1}
       : s == 8 ? Shape{2, 2, 3, 1}
       : s == 9 ? Shape{2, 3, 5, 0}
                : Shape{1, 2, 3, 0};
}

// Factor lists are expanded (a coefficient of 2 lists the species twice)
// and padded to MAXF entries per reaction.
constexpr int MAXF = 4;

}  // namespace crs
