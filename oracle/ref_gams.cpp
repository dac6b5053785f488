// ref_gams.cpp -- runs the reference's own GAMS frontend on a .gms file and
// prints the lowered Problem, for the parity tests of the Python frontend.
//
// TEST INFRASTRUCTURE ONLY.  Compiled by oracle/build_ref.sh together with
// the reference's source/gams/frontend.cpp, where it lies; the binary lands
// in oracle/_ref/.
//
// Output, one record per line (doubles as C99 hex floats):
//   ok <sense:min|max> <objvar_kept> <n_nodes> <n_vars> <n_constraints> <n_warnings>
//   node <op> <n_in> <in0> <in1> <constant> <var_index> <int_exp>
//   var <lb> <ub> <kind> <name>
//   obj <root>
//   con <root> <cmp> <rhs> <name>
// or, when the frontend rejects the file:
//   err <kind> <line>
#include <cstdio>
#include <iostream>
#include <string>

#include "cuminlp/gams.hpp"

using namespace cuminlp;

int main(int argc, char** argv)
{
  if (argc < 2) {
    std::cerr << "usage: ref_gams <model.gms>\n";
    return 2;
  }
  try {
    auto r = gams::parse_file<double>(argv[1], {});
    const auto& p = r.problem;
    const auto& nodes = p.graph.nodes;
    std::printf("ok %s %d %zu %zu %zu %zu\n", r.sense == gams::Sense::Maximise ? "max" : "min",
                r.objvar_kept ? 1 : 0, nodes.size(), p.box_bounds.size(), p.constraints.size(), r.warnings.size());
    for (const auto& nd : nodes) {
      const long in0 = nd.in.size() > 0 ? (long)nd.in[0] : -1;
      const long in1 = nd.in.size() > 1 ? (long)nd.in[1] : -1;
      double c = 0.0;
      unsigned long vi = 0;
      int ie = 0;
      if (nd.op == model::Op::Const) c = nd.payload.constant;
      if (nd.op == model::Op::Var) vi = nd.payload.var_index;
      if (nd.op == model::Op::PowN) ie = nd.payload.int_exp;
      std::printf("node %d %zu %ld %ld %a %lu %d\n", (int)nd.op, nd.in.size(), in0, in1, c, vi, ie);
    }
    for (std::size_t i = 0; i < p.box_bounds.size(); ++i)
      std::printf("var %a %a %d %s\n", p.box_bounds[i].lb, p.box_bounds[i].ub, (int)p.var_kinds[i],
                  i < r.var_names.size() ? r.var_names[i].c_str() : "?");
    std::printf("obj %zu\n", (std::size_t)p.objective_root);
    for (std::size_t i = 0; i < p.constraints.size(); ++i)
      std::printf("con %zu %d %a %s\n", (std::size_t)p.constraints[i].root_id, (int)p.constraints[i].cmp,
                  p.constraints[i].rhs, i < r.constraint_names.size() ? r.constraint_names[i].c_str() : "?");
  } catch (const gams::ParseError& e) {
    std::printf("err %d %d\n", (int)e.kind, e.line);
  }
  return 0;
}
