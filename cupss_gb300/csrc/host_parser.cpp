// Equation parser: string -> pres IR.
//
// Restates the grammar and lowering of the reference parser (src/parser.cpp),
// including its corner cases, so systems written for cuPSS lower to the same IR:
//   * spaces removed, split at the single '=' (:406-447)
//   * terms split at top-level '+'/'-' (:449-474), parentheses distributed (:477-545)
//   * factors split at top-level '*'; "a/b" becomes "a*1/b" (:547-589)
//   * factor kinds: q^n (q2n += n/2, integer division), iqx/iqy/iqz[^n], 1/q[^n],
//     field[^n], parameter, 1/parameter, number, 1/number (:125-267)
//   * LHS: "dt f" marks a dynamic field; remaining LHS terms are implicit, negated
//     for dynamic fields; the single trivial implicit {1,0,0,0,0,0} is dropped (:628-738)
//   * RHS terms grouped by their sorted field multiset (:701-725)
// Fatal errors throw cupssgb_host::ParseError (the reference prints and exits).
#include <algorithm>
#include <cctype>
#include <cstdlib>
#include <fstream>
#include <iostream>
#include <sstream>

#include "../../include/cupss.h"
#include "host_common.h"

using cupssgb_host::ParseError;

namespace {
bool starts_with(const std::string& s, const std::string& p) { return s.compare(0, p.size(), p) == 0; }

// "1/" marks inserted before every '/', as the reference does before splitting factors.
std::string mark_divisions(const std::string& t) {
  std::string out;
  out.reserve(t.size() + 8);
  for (char c : t) {
    if (c == '/') out += "*1";
    out += c;
  }
  return out;
}

std::string strip_sign(const std::string& t, bool* negative) {
  std::string s = t;
  if (negative) *negative = false;
  if (!s.empty() && s[0] == '+') s = s.substr(1);
  if (!s.empty() && s[0] == '-') {
    if (negative) *negative = true;
    s = s.substr(1);
  }
  return s;
}
}  // namespace

parser::parser(evolver* _system) : verbose(false), system(_system) {}

int parser::createFromFile(const std::string& file_name) {
  std::cout << "Trying to read system from " << file_name << std::endl;
  std::ifstream in(file_name);
  if (!in.is_open()) throw ParseError("cannot open system file " + file_name);
  int section = -1;   // 0 fields, 1 parameters, 2 equations
  std::vector<std::string> equations;
  std::string line;
  auto header = [](const std::string& l) -> int {
    if (starts_with(l, "Fields") || starts_with(l, "fields")) return 0;
    if (starts_with(l, "Parameters") || starts_with(l, "parameters")) return 1;
    if (starts_with(l, "Equations") || starts_with(l, "equations")) return 2;
    return -1;
  };
  while (std::getline(in, line)) {
    std::cout << line << std::endl;
    if (line.empty() || line[0] == '#') continue;
    const int h = header(line);
    if (h >= 0) {
      section = h;
      continue;
    }
    if (section == -1) {
      std::cout << "ERROR: reading file " << file_name << std::endl;
      std::cout << "First line must be either fields, parameters, or equations, it is:" << std::endl;
      std::cout << line << std::endl;
      return -1;
    }
    std::istringstream is(line);
    if (section == 0) {
      std::string name;
      int dyn, out;
      if (!(is >> name >> dyn >> out)) {
        std::cout << "Error reading field line: " << line << std::endl;
        std::cout << "Must be: field_name dynamic_value output" << std::endl;
        return -1;
      }
      std::cout << "Creating field: " << name << ", dynamic: " << dyn << std::endl;
      system->createField(name, dyn != 0);
      system->setOutputField(name, out);
    } else if (section == 1) {
      std::string name;
      float value;
      if (!(is >> name >> value)) {
        std::cout << "Error reading parameter line: " << line << std::endl;
        std::cout << "Must be: param_name value" << std::endl;
        return -1;
      }
      std::cout << "Creating parameter: " << name << " = " << value << std::endl;
      insert_parameter(name, value);
    } else {
      equations.push_back(line);
    }
  }
  for (const std::string& eq : equations) add_equation(eq);
  return 0;
}

int parser::insert_parameter(const std::string& name, float value) {
  if (exists_parameter(name)) {
    std::cout << "Duplicate parameter " << name << std::endl;
    return -1;
  }
  parameters[name] = value;
  return 0;
}

int parser::exists_parameter(const std::string& name) { return parameters.count(name) ? 1 : 0; }

int parser::is_number(const std::string& term) {
  std::string t = starts_with(term, "1/") ? term.substr(2) : term;
  size_t periods = std::count(t.begin(), t.end(), '.');
  if (periods > 1) throw ParseError("prefactor not a parameter and not a number: " + term);
  if (periods == 1) t.erase(t.find_last_of('.'), 1);
  for (char c : t)
    if (!std::isdigit((unsigned char)c)) return 0;
  return 1;
}

float parser::is_numerical_factor(const std::string& factor) {
  if (is_q2n_factor(factor)) return 1.0f;
  if (is_iq_factor(factor, "iqx") || is_iq_factor(factor, "iqy") || is_iq_factor(factor, "iqz") ||
      is_iq_factor(factor, "1/q"))
    return 1.0f;
  if (is_field(factor)) return 1.0f;
  const bool divides = starts_with(factor, "1/");
  const std::string f = divides ? factor.substr(2) : factor;
  if (exists_parameter(f)) return divides ? 1.0f / parameters[f] : parameters[f];
  if (is_number(f) && !f.empty()) {
    const float v = std::strtof(f.c_str(), nullptr);
    return divides ? 1.0f / v : v;
  }
  throw ParseError("parameter not found and not a number: " + factor);
}

int parser::is_field(const std::string& factor) {
  int power = 1;
  size_t caret = 0;
  for (size_t i = 0; i < factor.size(); ++i)
    if (factor[i] == '^') {
      power = std::atoi(factor.c_str() + i + 1);
      caret = i;
    }
  const std::string name = (power != 1) ? factor.substr(0, caret) : factor;
  for (field* f : system->fields)
    if (f->name == name) return power;
  return 0;
}

int parser::is_q2n_factor(const std::string& factor) {
  if (factor.size() < 3) return 0;
  if (factor[0] == 'q' && factor[1] == '^') {
    const std::string num = factor.substr(2);
    if (!is_number(num)) throw ParseError(num + " power of q not a number, missing *?");
    return std::atoi(num.c_str());
  }
  return 0;
}

int parser::is_iq_factor(const std::string& factor, const std::string& iq) {
  if (factor.size() < 3) return 0;
  if (factor.compare(0, 3, iq) != 0) return 0;
  if (factor.size() == 3) return 1;
  const std::string num = factor.size() > 4 ? factor.substr(4) : std::string();
  if (!is_number(num)) throw ParseError(num + " power of " + iq + " not a number, missing *?");
  return std::atoi(num.c_str());
}

std::string parser::extract_field_name(const std::string& t) {
  if (is_field(t) == 1) return t;
  size_t caret = 0;
  for (size_t i = 0; i < t.size(); ++i)
    if (t[i] == '^') caret = i;
  return t.substr(0, caret);
}

void parser::get_factors(const std::string& t, std::vector<std::string>& factors) {
  size_t start = 0;
  int opened = 0;
  for (size_t p = 0; p < t.size(); ++p) {
    if (t[p] == '(') opened = 1;
    if (t[p] == ')') opened = 0;
    if (t[p] == '*' && opened == 0) {
      factors.push_back(t.substr(start, p - start));
      start = p + 1;
    }
    if (p == t.size() - 1) factors.push_back(t.substr(start));
  }
}

std::string parser::get_field_name(const std::string& t) {
  std::vector<std::string> factors;
  get_factors(strip_sign(t, nullptr), factors);
  std::string name;
  for (const std::string& f : factors)
    if (is_field(f) > 0) name = f;
  return name;
}

int parser::number_of_fields(const std::string& t) {
  std::vector<std::string> factors;
  std::string s = t;
  if (!s.empty() && (s[0] == '+' || s[0] == '-')) s = s.substr(1);
  get_factors(s, factors);
  int n = 0;
  for (const std::string& f : factors) n += is_field(f);
  return n;
}

pres parser::add_noise(const std::string& eq_in) {
  std::string eq = eq_in;
  remove_spaces(eq);
  std::vector<std::string> factors;
  get_factors(eq, factors);
  pres p = {1.0f, 0, 0, 0, 0, 0};
  for (const std::string& f : factors) {
    p.preFactor *= is_numerical_factor(f);
    p.q2n += is_q2n_factor(f) / 2;
    p.invq += is_iq_factor(f, "1/q");
  }
  return p;
}

int parser::split_equation_sides(std::string input, std::string& lhs, std::string& rhs) {
  const size_t n = std::count(input.begin(), input.end(), '=');
  if (n != 1) throw ParseError("Error processing " + input + ": more than one equal sign");
  const size_t pos = input.find('=');
  lhs = input.substr(0, pos);
  rhs = (pos == input.size() - 1) ? std::string() : input.substr(pos + 1);
  return 0;
}

int parser::remove_spaces(std::string& input) {
  input.erase(std::remove(input.begin(), input.end(), ' '), input.end());
  return 0;
}

int parser::split_terms(std::string input, std::vector<std::string>& terms) {
  size_t cur = 0;
  int level = 0;
  for (size_t p = 0; p < input.size(); ++p) {
    if (input[p] == '(') ++level;
    if (input[p] == ')') --level;
    if (p > 0 && level == 0 && (input[p] == '+' || input[p] == '-')) {
      terms.push_back(input.substr(cur, p - cur));
      cur = p;
    }
  }
  terms.push_back(input.substr(cur));
  return 0;
}

int parser::expand_once(std::string input, std::vector<std::string>& terms) {
  int level = 0;
  bool found = false;
  size_t open = 0;
  for (size_t p = 0; p < input.size(); ++p) {
    if (input[p] == '(') {
      if (p > 0 && input[p - 1] == '/') throw ParseError("No dividing over parenthesis allowed!");
      found = true;
      ++level;
      if (level == 1) open = p;
    }
    if (input[p] == ')') --level;
    if (level == 0 && found) {
      std::vector<std::string> inner;
      split_terms(input.substr(open + 1, p - open - 1), inner);
      const std::string pre = input.substr(0, open);
      const std::string post = input.substr(p + 1);
      for (std::string t : inner) {
        std::string this_pre = pre;
        if (starts_with(t, "+")) t = t.substr(1);
        if (starts_with(t, "-")) {
          if (starts_with(this_pre, "-")) this_pre = "+" + this_pre.substr(1);
          else if (starts_with(this_pre, "+")) this_pre = "-" + pre.substr(1);
          else this_pre = "-" + this_pre;
          t = t.substr(1);
        }
        terms.push_back(this_pre + t + post);
      }
      return 1;
    }
  }
  return 0;
}

int parser::expand_all(std::vector<std::string>& terms) {
  for (size_t k = 0; k < terms.size();) {
    std::vector<std::string> sub;
    if (expand_once(terms[k], sub) > 0) {
      terms.erase(terms.begin() + k);
      terms.insert(terms.end(), sub.begin(), sub.end());
    } else {
      ++k;
    }
  }
  return 0;
}

pres parser::get_prefactor(const std::string& t_in) {
  pres p = {1.0f, 0, 0, 0, 0, 0};
  bool neg = false;
  const std::string t = mark_divisions(strip_sign(t_in, &neg));
  if (neg) p.preFactor = -1.0f;
  std::vector<std::string> factors;
  get_factors(t, factors);
  for (const std::string& f : factors) {
    if (is_field(f) > 0) continue;
    p.preFactor *= is_numerical_factor(f);
    p.q2n += is_q2n_factor(f) / 2;
    p.iqx += is_iq_factor(f, "iqx");
    p.iqy += is_iq_factor(f, "iqy");
    p.iqz += is_iq_factor(f, "iqz");
    p.invq += is_iq_factor(f, "1/q");
  }
  return p;
}

int parser::get_field_vector(const std::string& t_in, std::vector<std::string>& out) {
  const std::string t = mark_divisions(strip_sign(t_in, nullptr));
  std::vector<std::string> factors;
  get_factors(t, factors);
  for (const std::string& f : factors) {
    const int n = is_field(f);
    if (n > 0) {
      const std::string name = extract_field_name(f);
      for (int i = 0; i < n; ++i) out.push_back(name);
    }
  }
  return 0;
}

int parser::add_equation(const std::string& eq_in) {
  std::string eq = eq_in;
  remove_spaces(eq);
  if (verbose) std::cout << "Processing\n" << eq << "\n";
  std::string lhs, rhs;
  split_equation_sides(eq, lhs, rhs);
  std::vector<std::string> lhs_terms, rhs_terms;
  split_terms(lhs, lhs_terms);
  split_terms(rhs, rhs_terms);
  expand_all(lhs_terms);
  expand_all(rhs_terms);

  bool dynamic = false;
  std::string name;
  if (starts_with(lhs_terms[0], "dt")) {
    dynamic = true;
    name = lhs_terms[0].substr(2);
    if (!is_field(name)) throw ParseError("Field not found: " + name);
    if (is_field(name) > 1) throw ParseError("Nonlinearity in lhs: " + name);
    lhs_terms.erase(lhs_terms.begin());
  } else {
    if (number_of_fields(lhs_terms[0]) != 1)
      throw ParseError("Nonlinear term in left hand side: " + lhs_terms[0]);
    name = get_field_name(lhs_terms[0]);
  }
  auto it = system->fieldsMap.find(name);
  if (it == system->fieldsMap.end() || it->second == nullptr)
    throw ParseError("Field not found: " + name);
  field* target = it->second;

  std::vector<pres> implicits;
  for (const std::string& t : lhs_terms) {
    std::vector<std::string> fv;
    get_field_vector(t, fv);
    if (fv.size() != 1) throw ParseError("Nonlinear term in lhs");
    if (fv[0] != name) throw ParseError(name + " and " + fv[0] + " incompatible in lhs");
    pres p = get_prefactor(t);
    if (dynamic) p.preFactor *= -1.0f;
    implicits.push_back(p);
  }

  std::vector<std::vector<std::string>> groups;
  std::vector<std::vector<pres>> group_pres;
  std::vector<std::vector<std::string>> group_strings;
  for (const std::string& t : rhs_terms) {
    std::vector<std::string> fv;
    get_field_vector(t, fv);
    std::sort(fv.begin(), fv.end());
    const pres p = get_prefactor(t);
    bool hit = false;
    for (size_t k = 0; k < groups.size(); ++k) {
      if (groups[k] == fv) {
        hit = true;
        group_pres[k].push_back(p);
        group_strings[k].push_back(t);
      }
    }
    if (!hit) {
      groups.push_back(fv);
      group_pres.push_back({p});
      group_strings.push_back({t});
    }
  }
  for (const auto& kv : parameters) target->usedParameters[kv.first] = 0;
  const bool trivial = implicits.size() == 1 && implicits[0].preFactor == 1.0f && implicits[0].q2n == 0 &&
                       implicits[0].iqx == 0 && implicits[0].iqy == 0 && implicits[0].iqz == 0 &&
                       implicits[0].invq == 0;
  if (!trivial) {
    for (size_t i = 0; i < implicits.size(); ++i) {
      target->implicit.push_back(implicits[i]);
      target->addImplicitString(lhs_terms[i]);
      for (const auto& kv : parameters)
        if (isParameterInString(lhs_terms[i], kv.first)) target->usedParameters[kv.first] = 1;
    }
  }
  for (size_t i = 0; i < groups.size(); ++i) {
    system->createTerm(name, group_pres[i], groups[i]);
    term* tr = target->terms.back();
    tr->setPrefactorString(group_strings[i]);
    for (const auto& kv : parameters) tr->usedParameters[kv.first] = 0;
    for (const std::string& s : group_strings[i])
      for (const auto& kv : parameters)
        if (isParameterInString(s, kv.first)) tr->usedParameters[kv.first] = 1;
  }
  return 0;
}

void parser::writeParamsToFile(const std::string& file_name) {
  std::ofstream out(file_name);
  for (const auto& kv : parameters) out << kv.first << "\t" << kv.second << "\n";
}

float parser::getParameter(const std::string& name) {
  if (!exists_parameter(name)) throw ParseError("getParameter " + name + " not found");
  return parameters[name];
}

int parser::changeParameter(const std::string& name, float value) {
  if (!exists_parameter(name)) throw ParseError("changeParameter " + name + " not found");
  parameters[name] = value;
  return 0;
}

int parser::isParameterInString(const std::string& s, const std::string& param) {
  std::string local = s;
  if (!local.empty() && (local[0] == '+' || local[0] == '-')) local.erase(local.begin());
  std::replace(local.begin(), local.end(), '/', '*');
  std::vector<std::string> factors;
  get_factors(local, factors);
  int n = 0;
  for (const std::string& f : factors)
    if (f == param) ++n;
  return n;
}

int parser::recalculateImplicits(const std::vector<std::string>& strings, std::vector<pres>& out,
                                 int dynamic) {
  for (size_t i = 0; i < strings.size() && i < out.size(); ++i) {
    out[i] = get_prefactor(strings[i]);
    if (dynamic) out[i].preFactor *= -1.0f;
  }
  return 0;
}
