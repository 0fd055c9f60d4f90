// Oracle (test infrastructure only): the joint tree-contact solve.
// Placeholder until the tree-contact restatement lands: worlds whose
// contacts touch tree links are rejected.
#pragma once
#include <stdexcept>
#include "newt_world.hpp"

namespace oracle {

template <class R> void solve_tree_contacts(World<R>& w, const std::vector<Contact<R>>& tc, bool use_newton) {
  (void)w; (void)use_newton;
  if (!tc.empty()) throw std::runtime_error("tree contacts not supported by this oracle build");
}

}  // namespace oracle
