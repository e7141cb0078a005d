// The reference's circuit text format (docs/input_format.md): first line is
// the qubit count, then one "time gate qubits params" per line; "c q... gate"
// prefixes control qubits; "m q..." measures.  Validation follows
// lib/circuit_qsim_parser.h:52-153: qubit indices in range and distinct,
// times of gates on the same qubit ordered, nothing crossing a measurement
// time boundary.  Angles are read as float, as the reference parses them
// into fp_type = float.

#include <algorithm>
#include <cctype>
#include <sstream>

#include "engine.h"

namespace qsg {
namespace host {

namespace {

struct NamedArity {
  const char* name;
  unsigned nq;
  unsigned np;
};

const NamedArity kGates[] = {
    {"p", 0, 1},      {"id1", 1, 0},  {"h", 1, 0},      {"t", 1, 0},
    {"x", 1, 0},      {"y", 1, 0},    {"z", 1, 0},      {"x_1_2", 1, 0},
    {"y_1_2", 1, 0},  {"rx", 1, 1},   {"ry", 1, 1},     {"rz", 1, 1},
    {"rxy", 1, 2},    {"hz_1_2", 1, 0}, {"s", 1, 0},    {"id2", 2, 0},
    {"cz", 2, 0},     {"cnot", 2, 0}, {"cx", 2, 0},     {"sw", 2, 0},
    {"is", 2, 0},     {"fs", 2, 2},   {"cp", 2, 1},
};

const NamedArity* find_gate(const std::string& name) {
  for (const auto& g : kGates)
    if (name == g.name) return &g;
  return nullptr;
}

bool distinct_in_range(const std::vector<unsigned>& qs, unsigned n) {
  for (size_t i = 0; i < qs.size(); ++i) {
    if (qs[i] >= n) return false;
    for (size_t j = 0; j < i; ++j)
      if (qs[i] == qs[j]) return false;
  }
  return true;
}

}  // namespace

bool parse_qsim_text(const std::string& text, unsigned maxtime, Circuit* out,
                     std::string* err) {
  out->num_qubits = 0;
  out->ops.clear();
  std::istringstream in(text);
  std::string line;
  unsigned lineno = 0, max_time = 0, prev_meas_time = 0;
  std::vector<long long> last_time;
  auto fail = [&](const char* why) {
    if (err) {
      std::ostringstream o;
      o << why << " in line " << lineno;
      *err = o.str();
    }
    return false;
  };
  while (std::getline(in, line)) {
    ++lineno;
    if (line.empty() || line[0] == '#') continue;
    std::istringstream ss(line);
    if (out->num_qubits == 0) {
      long long n = 0;
      ss >> n;
      if (n <= 0 || n > 63) return fail("invalid number of qubits");
      out->num_qubits = unsigned(n);
      last_time.assign(out->num_qubits, -1);
      continue;
    }
    unsigned time;
    std::string name;
    if (!(ss >> time >> name)) return fail("invalid gate");
    if (time > maxtime) break;
    std::vector<unsigned> ctrl;
    if (name == "c") {
      while (ss >> std::ws && std::isdigit(ss.peek())) {
        unsigned q;
        ss >> q;
        ctrl.push_back(q);
      }
      if (ctrl.empty() || !(ss >> name)) return fail("invalid controlled gate");
      if (name == "m") return fail("measurement gate cannot be controlled");
    }
    Op op;
    if (name == "m") {
      std::vector<unsigned> qs;
      unsigned q;
      while (ss >> q) qs.push_back(q);
      if (!ss.eof() || qs.empty() || !distinct_in_range(qs, out->num_qubits))
        return fail("invalid measurement");
      op.kind = OpKind::kMeasure;
      op.time = time;
      std::sort(qs.begin(), qs.end());
      op.qs = qs;
    } else {
      const NamedArity* g = find_gate(name);
      if (!g) return fail("unknown gate");
      std::vector<unsigned> qs(g->nq);
      std::vector<double> ps(g->np);
      for (auto& q : qs)
        if (!(ss >> q)) return fail("invalid gate");
      for (auto& p : ps) {
        float f;
        if (!(ss >> f)) return fail("invalid gate parameter");
        p = f;
      }
      std::string extra;
      if (ss >> extra) return fail("trailing characters");
      if (!distinct_in_range(qs, out->num_qubits)) return fail("invalid qubit");
      if (!named_gate(name, time, qs, ps, &op)) return fail("invalid gate");
      if (!ctrl.empty()) {
        std::vector<unsigned> all = qs;
        all.insert(all.end(), ctrl.begin(), ctrl.end());
        if (!distinct_in_range(all, out->num_qubits))
          return fail("invalid control qubit");
        std::sort(ctrl.begin(), ctrl.end());
        op.kind = OpKind::kControlled;
        op.cqs = ctrl;
        op.cvals = (uint64_t{1} << ctrl.size()) - 1;  // all controls on |1>
      }
    }
    const bool is_meas = op.kind == OpKind::kMeasure;
    if (time < prev_meas_time || (is_meas && time < max_time))
      return fail("operation crosses a measurement time boundary");
    if (is_meas) prev_meas_time = time;
    auto check_order = [&](const std::vector<unsigned>& qs) {
      for (unsigned q : qs) {
        if (last_time[q] >= 0 && (long long)time < last_time[q]) return false;
      }
      for (unsigned q : qs) last_time[q] = time;
      return true;
    };
    if (!check_order(op.qs) || !check_order(op.cqs))
      return fail("operation is out of time order");
    max_time = std::max(max_time, time);
    out->ops.push_back(std::move(op));
  }
  if (out->num_qubits == 0) return fail("empty circuit");
  return true;
}

}  // namespace host
}  // namespace qsg
