// Per-member parsing and batch-solver construction for the batched forms.
#include "host_ir.h"

#include <sstream>
#include <stdexcept>

#include "../../include/cupss.h"
#include "host_common.h"

namespace cupssgb_host {

void ok(int rc) {
  if (rc < 0) throw CapiError(rc, cupssgb_last_error());
}

namespace {
cupssgb_pres to_c(const pres& p) { return {p.preFactor, p.q2n, p.iqx, p.iqy, p.iqz, p.invq}; }
}  // namespace

std::vector<IrField> parse_system(const std::vector<SystemOp>& ops, const std::map<std::string, float>& values) {
  // The parser works on an evolver's fields; the grid does not enter the IR, so a
  // one-point evolver (no device work before prepareProblem) is enough.
  evolver ev(true, 1, 1, 1, 1.f, 1.f, 1.f, 1.f, 1);
  ev.setThrowOnError(true);
  for (const SystemOp& op : ops) {
    switch (op.kind) {
      case SystemOp::kField:
        if (ev.createField(op.a, op.dynamic) != 0) throw ParseError("field " + op.a + " declared twice");
        break;
      case SystemOp::kParameter: {
        auto it = values.find(op.a);
        ev.addParameter(op.a, it != values.end() ? it->second : op.value);
        break;
      }
      case SystemOp::kEquation:
        ev.addEquation(op.a);
        break;
      case SystemOp::kNoise:
        if (ev.addNoise(op.a, op.b) != 0) throw ParseError("noise on unknown field " + op.a);
        break;
    }
  }
  std::vector<IrField> ir;
  for (field* f : ev.fields) {
    IrField F;
    F.name = f->name;
    F.dynamic = f->dynamic;
    for (const pres& p : f->implicit) F.implicit.push_back(to_c(p));
    for (term* t : f->terms) {
      IrTerm T;
      for (field* g : t->product) T.product.push_back(ev.existsField(g->name));
      for (const pres& p : t->prefactors_h) T.pres.push_back(to_c(p));
      F.terms.push_back(T);
    }
    F.noisy = f->isNoisy;
    if (F.noisy) F.noise = to_c(f->noise_amplitude);
    ir.push_back(F);
  }
  return ir;
}

std::string structure_key(const std::vector<IrField>& ir) {
  std::ostringstream os;
  auto mono = [&](const cupssgb_pres& p) {
    os << "(" << p.q2n << "," << p.iqx << "," << p.iqy << "," << p.iqz << "," << p.invq << ")";
  };
  for (const IrField& f : ir) {
    os << "F" << (f.dynamic ? 1 : 0) << "[";
    for (const cupssgb_pres& p : f.implicit) mono(p);
    os << "]";
    for (const IrTerm& t : f.terms) {
      os << "T{";
      for (int g : t.product) os << g << ",";
      os << "}";
      for (const cupssgb_pres& p : t.pres) mono(p);
    }
    if (f.noisy) {
      os << "N";
      mono(f.noise);
    }
    os << ";";
  }
  return os.str();
}

cupssgb_solver* create_solver(const std::vector<IrField>& ir, int sx, int sy, int sz, float dx, float dy, float dz,
                              float dt) {
  cupssgb_solver* s = nullptr;
  ok(cupssgb_solver_create(sx, sy, sz, dx, dy, dz, dt, &s));
  try {
    for (const IrField& f : ir) ok(cupssgb_solver_add_field(s, f.dynamic ? 1 : 0));
    for (size_t i = 0; i < ir.size(); ++i) {
      const IrField& f = ir[i];
      ok(cupssgb_solver_set_implicit(s, (int)i, f.implicit.data(), (int)f.implicit.size()));
      for (const IrTerm& t : f.terms)
        ok(cupssgb_solver_add_term(s, (int)i, t.product.data(), (int)t.product.size(), t.pres.data(),
                                   (int)t.pres.size()));
      if (f.noisy) ok(cupssgb_solver_set_noise(s, (int)i, &f.noise));
    }
  } catch (...) {
    cupssgb_solver_destroy(s);
    throw;
  }
  return s;
}

void set_member(cupssgb_solver* s, int m, const std::vector<IrField>& ir, unsigned long long seed) {
  for (size_t i = 0; i < ir.size(); ++i) {
    const IrField& f = ir[i];
    ok(cupssgb_solver_set_member_implicit(s, m, (int)i, f.implicit.data(), (int)f.implicit.size()));
    for (size_t t = 0; t < f.terms.size(); ++t)
      ok(cupssgb_solver_set_member_term_pres(s, m, (int)i, (int)t, f.terms[t].pres.data(),
                                            (int)f.terms[t].pres.size()));
    if (f.noisy) ok(cupssgb_solver_set_member_noise(s, m, (int)i, &f.noise));
  }
  ok(cupssgb_solver_set_member_seed(s, m, seed));
}

}  // namespace cupssgb_host
