// ensemble: batched independent solves on the solver-level C-ABI (see
// include/cupss/ensemble.h).  Errors throw std::runtime_error / ParseError.
#include "../../include/cupss/ensemble.h"

#include <cstdlib>
#include <map>
#include <sstream>
#include <stdexcept>
#include <tuple>
#include <vector>

#include "../../include/cupss_gb300.h"
#include "host_ir.h"

using cupssgb_host::IrField;
using cupssgb_host::ok;
using cupssgb_host::SystemOp;

struct ensemble::Impl {
  struct Member {
    int sx, sy, sz;
    float dx, dy, dz, dt;
    unsigned long long seed;
    std::map<std::string, float> values;
    int group = -1, slot = -1;
  };
  struct Group {
    cupssgb_solver* solver = nullptr;
    int sx, sy, sz;
    float dt;
    std::vector<int> members;
  };
  std::vector<SystemOp> ops;
  std::vector<std::string> fields, params;
  std::vector<Member> members;
  std::vector<Group> groups;
  bool prepared = false;
  // every group stepped by one fused launch per kernel (1D/2D grids of one structure);
  // null when the groups do not qualify or CUPSSGB_FUSE=0
  cupssgb_multi* multi = nullptr;
  std::string multi_why;
  bool multi_fused = false;   // the multi stepper runs the fused launches (else each group alone)

  int field_index(const std::string& name) const {
    for (size_t i = 0; i < fields.size(); ++i)
      if (fields[i] == name) return (int)i;
    throw std::runtime_error("unknown field " + name);
  }
  const Member& member(int m) const {
    if (m < 0 || m >= (int)members.size()) throw std::runtime_error("bad member index");
    return members[m];
  }
  void before_prepare(const char* what) const {
    if (prepared) throw std::runtime_error(std::string(what) + " after prepare");
  }
};

ensemble::ensemble() : impl_(new Impl) {}

ensemble::~ensemble() {
  if (impl_->multi) cupssgb_multi_destroy(impl_->multi);
  for (auto& g : impl_->groups)
    if (g.solver) cupssgb_solver_destroy(g.solver);
  delete impl_;
}

int ensemble::createField(const std::string& name, bool dynamic) {
  impl_->before_prepare("createField");
  for (const std::string& f : impl_->fields)
    if (f == name) throw std::runtime_error("field " + name + " declared twice");
  SystemOp op{SystemOp::kField, name, "", 0.f, dynamic};
  impl_->ops.push_back(op);
  impl_->fields.push_back(name);
  return 0;
}

int ensemble::addParameter(const std::string& name, float value) {
  impl_->before_prepare("addParameter");
  SystemOp op{SystemOp::kParameter, name, "", value, false};
  impl_->ops.push_back(op);
  impl_->params.push_back(name);
  return 0;
}

int ensemble::addEquation(const std::string& equation) {
  impl_->before_prepare("addEquation");
  SystemOp op{SystemOp::kEquation, equation, "", 0.f, false};
  impl_->ops.push_back(op);
  return 0;
}

int ensemble::addNoise(const std::string& field, const std::string& amplitude) {
  impl_->before_prepare("addNoise");
  impl_->field_index(field);
  SystemOp op{SystemOp::kNoise, field, amplitude, 0.f, false};
  impl_->ops.push_back(op);
  return 0;
}

int ensemble::addMember(int sx, int sy, int sz, float dx, float dy, float dz, float dt, unsigned long long seed) {
  impl_->before_prepare("addMember");
  Impl::Member m;
  m.sx = sx;
  m.sy = sy;
  m.sz = sz;
  m.dx = dx;
  m.dy = dy;
  m.dz = dz;
  m.dt = dt;
  m.seed = seed;
  impl_->members.push_back(m);
  return (int)impl_->members.size() - 1;
}

int ensemble::setMemberParameter(int member, const std::string& name, float value) {
  impl_->before_prepare("setMemberParameter");
  impl_->member(member);
  bool known = false;
  for (const std::string& p : impl_->params) known = known || p == name;
  if (!known) throw std::runtime_error("unknown parameter " + name);
  impl_->members[member].values[name] = value;
  return 0;
}

void ensemble::prepare() {
  Impl& I = *impl_;
  I.before_prepare("prepare");
  if (I.members.empty()) throw std::runtime_error("ensemble without members");
  // parse every member; group by grid, cell, time step and equation structure
  std::vector<std::vector<IrField>> irs(I.members.size());
  std::map<std::tuple<int, int, int, float, float, float, float, std::string>, int> gid;
  for (size_t m = 0; m < I.members.size(); ++m) {
    Impl::Member& M = I.members[m];
    irs[m] = cupssgb_host::parse_system(I.ops, M.values);
    auto key = std::make_tuple(M.sx, M.sy, M.sz, M.dx, M.dy, M.dz, M.dt, cupssgb_host::structure_key(irs[m]));
    auto it = gid.find(key);
    if (it == gid.end()) {
      Impl::Group g;
      g.sx = M.sx;
      g.sy = M.sy;
      g.sz = M.sz;
      g.dt = M.dt;
      I.groups.push_back(g);
      it = gid.emplace(key, (int)I.groups.size() - 1).first;
    }
    M.group = it->second;
    M.slot = (int)I.groups[M.group].members.size();
    I.groups[M.group].members.push_back((int)m);
  }
  for (Impl::Group& g : I.groups) {
    const Impl::Member& M0 = I.members[g.members[0]];
    g.solver = cupssgb_host::create_solver(irs[g.members[0]], g.sx, g.sy, g.sz, M0.dx, M0.dy, M0.dz, g.dt);
    ok(cupssgb_solver_set_members(g.solver, (int)g.members.size()));
    for (size_t k = 0; k < g.members.size(); ++k)
      cupssgb_host::set_member(g.solver, (int)k, irs[g.members[k]], I.members[g.members[k]].seed);
    ok(cupssgb_solver_prepare(g.solver));
  }
  // one launch per kernel and step across every grid size, where the groups allow it
  // (CUPSSGB_FUSE=1: always fused; =0: never; unset: the faster form, timed here on the
  // zeroed buffers of the fresh groups)
  const char* fe = std::getenv("CUPSSGB_FUSE");
  const std::string fuse = fe ? fe : "";
  if (I.groups.size() < 2) {
    I.multi_why = "one grid class: stepped by its own tuned graphs";
  } else if (fuse != "0") {
    std::vector<cupssgb_solver*> sv;
    for (Impl::Group& g : I.groups) sv.push_back(g.solver);
    char why[256] = {0};
    if (cupssgb_multi_check(sv.data(), (int)sv.size(), why, (int)sizeof(why)) == 0) {
      ok(cupssgb_multi_create(sv.data(), (int)sv.size(), &I.multi));
      I.multi_fused = true;
      if (fuse != "1") {
        const int rc = cupssgb_multi_choose(I.multi);
        ok(rc);
        I.multi_fused = rc == 1;
      }
    } else {
      I.multi_why = why;
    }
  } else {
    I.multi_why = "CUPSSGB_FUSE=0";
  }
  I.prepared = true;
}

int ensemble::setReal(int member, const std::string& field, const float* host_real) {
  Impl& I = *impl_;
  if (!I.prepared) throw std::runtime_error("setReal before prepare");
  const Impl::Member& M = I.member(member);
  ok(cupssgb_solver_set_real_member(I.groups[M.group].solver, I.field_index(field), M.slot, host_real));
  return 0;
}

int ensemble::advance(int nsteps) {
  Impl& I = *impl_;
  if (!I.prepared) throw std::runtime_error("advance before prepare");
  if (I.multi) {
    // one launch per kernel and step over every group; the groups' streams wait for it
    ok(cupssgb_multi_advance(I.multi, nsteps));
  } else {
    // each group queues its steps on its own stream; they run concurrently
    for (Impl::Group& g : I.groups) ok(cupssgb_solver_advance(g.solver, nsteps));
  }
  for (Impl::Group& g : I.groups) ok(cupssgb_solver_synchronize(g.solver));
  return 0;
}

int ensemble::getReal(int member, const std::string& field, float* host_real) {
  Impl& I = *impl_;
  if (!I.prepared) throw std::runtime_error("getReal before prepare");
  const Impl::Member& M = I.member(member);
  ok(cupssgb_solver_get_real_member(I.groups[M.group].solver, I.field_index(field), M.slot, host_real));
  return 0;
}

int ensemble::members() const { return (int)impl_->members.size(); }
int ensemble::groups() const { return (int)impl_->groups.size(); }

long long ensemble::deviceBytes() const {
  long long b = 0;
  for (const auto& g : impl_->groups) b += cupssgb_solver_device_bytes(g.solver);
  return b;
}

long long ensemble::launches() const {
  long long n = 0;
  for (const auto& g : impl_->groups) n += cupssgb_solver_launch_count(g.solver);
  if (impl_->multi) n += cupssgb_multi_launch_count(impl_->multi);
  return n;
}

bool ensemble::fused() const { return impl_->multi != nullptr && impl_->multi_fused; }

std::string ensemble::describe() const {
  std::ostringstream os;
  os << "[";
  for (size_t i = 0; i < impl_->groups.size(); ++i) {
    const auto& g = impl_->groups[i];
    std::string tune;
    if (g.solver) {
      const int n = cupssgb_solver_tune_report(g.solver, nullptr, 0);
      tune.assign(n > 0 ? n : 0, '\0');
      if (n > 0) {
        std::vector<char> buf(n + 1);
        cupssgb_solver_tune_report(g.solver, buf.data(), n + 1);
        tune = buf.data();
      }
    }
    os << (i ? ", " : "") << "{\"grid\": [" << g.sx << ", " << g.sy << ", " << g.sz << "], \"dt\": " << g.dt
       << ", \"members\": " << g.members.size() << ", \"tune\": " << (tune.empty() ? "{}" : tune) << "}";
  }
  os << "]";
  if (impl_->multi) {
    const int n = cupssgb_multi_describe(impl_->multi, nullptr, 0);
    std::vector<char> buf(n + 1);
    cupssgb_multi_describe(impl_->multi, buf.data(), n + 1);
    return "{\"groups\": " + os.str() + ", \"fused\": " + buf.data() + "}";
  }
  return "{\"groups\": " + os.str() + ", \"fused\": null, \"why_not_fused\": \"" + impl_->multi_why + "\"}";
}
