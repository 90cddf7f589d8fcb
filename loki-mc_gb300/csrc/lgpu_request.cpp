// lgpu_request.cpp - swarm jobs from the reference's own input files (the
// lgpu_request_* entry points of include/loki_gpu.h).
//
// A serving client holds what a LoKI-MC user holds: a setup file (.in) and
// the LXCat files it names. This front end turns their texts into the jobs of
// lgpu_server_submit without the reference's host code, at the rate requests
// arrive (microseconds to milliseconds per request, no files touched):
//
//  * the setup file's indentation tree (Parse.C:611-700 reads the same
//    layout): "key: value", "key:" sections, "- item" lists, '%' comments;
//    values are arithmetic expressions (the reference hands them to its
//    expression parser, Parse.C:727-745) or vectors "[a, b, ...]",
//    "logspace(a, b, n)", "linspace(a, b, n)"; one working condition may be a
//    vector and makes one job per entry (Setup.h:166-181);
//  * the LXCat files (Parse.C:43-125): a PROCESS line, the parameter line with
//    "E = x eV" (the threshold; "m/M = x" for Elastic), the bracketed
//    description "[e + T -> e + P, Type(, integral|momentum-transfer)]"
//    (Parse.C:127-295) and the two-column data between dashed lines;
//  * gas and state properties (Setup.h:460-580): masses, fractions, OPB
//    parameters, state energies, statistical weights and populations, given
//    as values or as "boltzmannPopulation@T" over a family "G(X,v=*)"
//    (StatePropertyFunctions.h:172-197); the relative density of a state is
//    the gas fraction times the populations down its hierarchy (State.h:72-85);
//  * anisotropic scattering "group;gas;type;law;params" lines (Setup.h:351-459);
//  * the flattening of BoltzmannMC.C:29-271 into lgpu_process arrays: every
//    non-Effective collision once, a reversible one followed by its
//    superelastic copy (weight g_target / g_product), raw cross sections
//    clipped at the threshold (BoltzmannMC.C:139-147, Collision.C:40-43).
//
// Not covered (an error names the key): momentum-transfer cross sections of
// a process with an anisotropic law (the reference converts them with an
// angular integration, Collision.C:127-199), per-collision anisotropy lines,
// state properties other than energy, statistical weight and population.
#include <array>
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/loki_gpu.h"

namespace {

constexpr double kBoltzmann = 1.38064852e-23;  // Constant.h:8
constexpr double kElectronCharge = 1.6021766208e-19;
constexpr double kElectronMass = 9.10938356e-31;

struct Error : std::runtime_error {
  using std::runtime_error::runtime_error;
};

std::string trim(const std::string& s) {
  size_t a = 0, b = s.size();
  while (a < b && std::isspace((unsigned char)s[a])) ++a;
  while (b > a && std::isspace((unsigned char)s[b - 1])) --b;
  return s.substr(a, b - a);
}

std::string no_spaces(const std::string& s) {
  std::string o;
  for (char c : s)
    if (!std::isspace((unsigned char)c)) o += c;
  return o;
}

std::vector<std::string> split_top(const std::string& s, char sep) {
  std::vector<std::string> out;
  int depth = 0;
  std::string cur;
  for (char c : s) {
    if (c == '(' || c == '[') ++depth;
    if (c == ')' || c == ']') --depth;
    if (c == sep && depth == 0) {
      out.push_back(cur);
      cur.clear();
    } else {
      cur += c;
    }
  }
  out.push_back(cur);
  return out;
}

// ---------------------------------------------------------------- expressions
// + - * / ^, unary signs, parentheses, numbers, pi, and sqrt exp log log10
// sin cos tan abs.
class Expr {
 public:
  explicit Expr(const std::string& s) : s_(s) {}
  double eval() {
    const double v = sum();
    skip();
    if (i_ != s_.size()) throw Error("cannot read the expression '" + s_ + "'");
    return v;
  }

 private:
  std::string s_;
  size_t i_ = 0;
  void skip() {
    while (i_ < s_.size() && std::isspace((unsigned char)s_[i_])) ++i_;
  }
  bool take(char c) {
    skip();
    if (i_ < s_.size() && s_[i_] == c) {
      ++i_;
      return true;
    }
    return false;
  }
  double sum() {
    double v = product();
    for (;;) {
      if (take('+')) v += product();
      else if (take('-')) v -= product();
      else return v;
    }
  }
  double product() {
    double v = unary();
    for (;;) {
      if (take('*')) v *= unary();
      else if (take('/')) v /= unary();
      else return v;
    }
  }
  double unary() {
    if (take('-')) return -unary();
    if (take('+')) return unary();
    return power();
  }
  double power() {
    const double b = primary();
    if (take('^')) return std::pow(b, unary());
    return b;
  }
  double primary() {
    skip();
    if (take('(')) {
      const double v = sum();
      if (!take(')')) throw Error("missing ')' in '" + s_ + "'");
      return v;
    }
    if (i_ < s_.size() && (std::isdigit((unsigned char)s_[i_]) || s_[i_] == '.')) {
      const char* p = s_.c_str() + i_;
      char* end = nullptr;
      const double v = std::strtod(p, &end);
      i_ += (size_t)(end - p);
      return v;
    }
    std::string name;
    while (i_ < s_.size() && (std::isalnum((unsigned char)s_[i_]) || s_[i_] == '_')) name += s_[i_++];
    if (name == "pi") return M_PI;
    if (name.empty()) throw Error("cannot read the expression '" + s_ + "'");
    if (!take('(')) throw Error("unknown name '" + name + "' in '" + s_ + "'");
    const double a = sum();
    if (!take(')')) throw Error("missing ')' in '" + s_ + "'");
    if (name == "sqrt") return std::sqrt(a);
    if (name == "exp") return std::exp(a);
    if (name == "log") return std::log(a);
    if (name == "log10") return std::log10(a);
    if (name == "sin") return std::sin(a);
    if (name == "cos") return std::cos(a);
    if (name == "tan") return std::tan(a);
    if (name == "abs") return std::fabs(a);
    throw Error("unknown function '" + name + "' in '" + s_ + "'");
  }
};

double value_of(const std::string& s) { return Expr(s).eval(); }

// A scalar, "[a, b, ...]", "logspace(a, b, n)" or "linspace(a, b, n)".
std::vector<double> values_of(const std::string& s0) {
  const std::string s = trim(s0);
  std::vector<double> out;
  if (!s.empty() && s.front() == '[' && s.back() == ']') {
    for (const std::string& t : split_top(s.substr(1, s.size() - 2), ',')) out.push_back(value_of(t));
    return out;
  }
  for (const char* fn : {"logspace(", "linspace("}) {
    if (s.rfind(fn, 0) == 0 && s.back() == ')') {
      const auto a = split_top(s.substr(9, s.size() - 10), ',');
      if (a.size() != 3) throw Error("'" + s + "' needs three arguments");
      const double lo = value_of(a[0]), hi = value_of(a[1]);
      const int n = (int)value_of(a[2]);
      for (int k = 0; k < n; ++k) {
        const double x = n > 1 ? lo + (hi - lo) * k / (n - 1) : lo;
        out.push_back(fn[1] == 'o' ? std::pow(10.0, x) : x);
      }
      return out;
    }
  }
  out.push_back(value_of(s));
  return out;
}

// ------------------------------------------------------------------ setup tree
struct Node {
  std::string value;
  std::vector<std::string> items;
  std::vector<std::pair<std::string, std::unique_ptr<Node>>> children;
  const Node* child(const std::string& k) const {
    for (auto& c : children)
      if (c.first == k) return c.second.get();
    return nullptr;
  }
};

std::unique_ptr<Node> read_setup(const std::string& text) {
  auto root = std::make_unique<Node>();
  std::vector<std::pair<int, Node*>> stack{{-1, root.get()}};
  size_t pos = 0;
  int line_no = 0;
  while (pos <= text.size()) {
    size_t e = text.find('\n', pos);
    if (e == std::string::npos) e = text.size();
    std::string line = text.substr(pos, e - pos);
    pos = e + 1;
    ++line_no;
    const size_t pc = line.find('%');
    if (pc != std::string::npos) line = line.substr(0, pc);
    if (trim(line).empty()) continue;
    int indent = 0;
    while (indent < (int)line.size() && (line[indent] == ' ' || line[indent] == '\t')) ++indent;
    const std::string body = trim(line);
    while (stack.size() > 1 && stack.back().first >= indent) stack.pop_back();
    Node* parent = stack.back().second;
    if (body[0] == '-') {
      parent->items.push_back(trim(body.substr(1)));
      continue;
    }
    const size_t colon = body.find(':');
    if (colon == std::string::npos) throw Error("setup line " + std::to_string(line_no) + ": no ':' in '" + body + "'");
    auto n = std::make_unique<Node>();
    n->value = trim(body.substr(colon + 1));
    Node* raw = n.get();
    parent->children.emplace_back(trim(body.substr(0, colon)), std::move(n));
    stack.push_back({indent, raw});
  }
  return root;
}

// "name = value" items of a list
std::vector<std::pair<std::string, std::string>> assignments(const Node* n) {
  std::vector<std::pair<std::string, std::string>> out;
  if (!n) return out;
  for (const std::string& it : n->items) {
    // the '=' outside the state name's parentheses ("X2(X,v=0) = 0.5")
    size_t eq = std::string::npos;
    int depth = 0;
    for (size_t k = 0; k < it.size() && eq == std::string::npos; ++k) {
      if (it[k] == '(') ++depth;
      else if (it[k] == ')') --depth;
      else if (it[k] == '=' && depth == 0) eq = k;
    }
    if (eq == std::string::npos) throw Error("expected 'name = value' in '" + it + "'");
    out.emplace_back(no_spaces(it.substr(0, eq)), trim(it.substr(eq + 1)));
  }
  return out;
}

// ------------------------------------------------------------------- LXCat
struct Coll {
  std::string type, target, product;
  bool reverse = false, integral = true;
  double threshold = 0, mass_ratio = 0;
  std::vector<double> e, v;
};

std::string gas_of(const std::string& state) {
  std::string g = state.substr(0, state.find('('));
  const size_t caret = g.find('^');
  return caret == std::string::npos ? g : g.substr(0, caret);
}

// the non-electron species of one side of a collision ("e+X2(X)" -> X2(X))
std::vector<std::string> species(const std::string& side) {
  std::vector<std::string> out;
  for (const std::string& t : split_top(side, '+')) {
    std::string s = t;
    while (!s.empty() && std::isdigit((unsigned char)s[0])) s.erase(0, 1);  // stoichiometric coefficient
    if (!s.empty() && s != "e" && s != "E") out.push_back(s);
  }
  return out;
}

void read_lxcat(const std::string& name, const std::string& text, std::vector<Coll>& out) {
  std::vector<std::string> lines;
  size_t pos = 0;
  while (pos <= text.size()) {
    size_t e = text.find('\n', pos);
    if (e == std::string::npos) e = text.size();
    std::string l = text.substr(pos, e - pos);
    if (!l.empty() && l.back() == '\r') l.pop_back();
    lines.push_back(l);
    pos = e + 1;
  }
  for (size_t k = 0; k < lines.size(); ++k) {
    if (lines[k].find("PROCESS:") == std::string::npos) continue;
    const std::string process = lines[k];
    if (k + 2 >= lines.size()) throw Error(name + ": truncated process '" + process + "'");
    const std::string param = lines[k + 1], descr = lines[k + 2];
    Coll c;
    const size_t eq = param.find("E =");
    const size_t ev = param.find("eV");
    if (eq != std::string::npos && ev != std::string::npos && ev > eq) c.threshold = value_of(param.substr(eq + 3, ev - eq - 3));
    const size_t mm = param.find("m/M =");
    if (mm != std::string::npos) c.mass_ratio = value_of(param.substr(mm + 5, param.find_first_of(",\n", mm) - mm - 5));
    const std::string d = no_spaces(descr);
    const size_t lb = d.find('['), rb = d.rfind(']');
    if (lb == std::string::npos || rb == std::string::npos || rb < lb)
      throw Error(name + ": no [collision, type] description after '" + process + "'");
    std::vector<std::string> parts = split_top(d.substr(lb + 1, rb - lb - 1), ',');
    std::string sub;
    std::string last = parts.back();
    std::string lower = last;
    for (char& ch : lower) ch = (char)std::tolower((unsigned char)ch);
    if (lower == "integral" || lower == "momentum-transfer") {
      sub = lower;
      parts.pop_back();
      last = parts.back();
    }
    c.type = last;
    static const char* kTypes[] = {"Elastic", "Effective", "Attachment", "Ionization", "Excitation", "Vibrational",
                                   "Rotational"};
    bool known = false;
    for (const char* t : kTypes) known |= c.type == t;
    if (!known) throw Error(name + ": unknown collision type '" + c.type + "' in '" + descr + "'");
    if (sub.empty()) sub = (c.type == "Elastic" || c.type == "Effective") ? "momentum-transfer" : "integral";
    c.integral = sub == "integral";
    if (c.type != "Elastic" && c.type != "Effective" && eq == std::string::npos)
      throw Error(name + ": no threshold 'E = x eV' on the line after '" + process + "'");
    parts.pop_back();
    std::string coll;
    for (size_t q = 0; q < parts.size(); ++q) coll += (q ? "," : "") + parts[q];
    size_t arrow = coll.find("<->");
    size_t alen = 3;
    if (arrow != std::string::npos) c.reverse = true;
    else if ((arrow = coll.find("->")) != std::string::npos) alen = 2;
    else throw Error(name + ": no '->' in '" + descr + "'");
    const auto tgt = species(coll.substr(0, arrow));
    const auto prd = species(coll.substr(arrow + alen));
    if (tgt.size() != 1) throw Error(name + ": expected one target in '" + descr + "'");
    c.target = tgt[0];
    c.product = prd.empty() ? tgt[0] : prd[0];
    size_t j = k + 3;
    while (j < lines.size() && lines[j].find("-----") == std::string::npos) ++j;
    for (++j; j < lines.size() && lines[j].find("-----") == std::string::npos; ++j) {
      const std::string t = trim(lines[j]);
      if (t.empty()) continue;
      char* end = nullptr;
      const double x = std::strtod(t.c_str(), &end);
      char* end2 = nullptr;
      const double y = std::strtod(end, &end2);
      if (end == t.c_str() || end2 == end || !trim(end2).empty())
        throw Error(name + ": bad cross-section line '" + t + "' after '" + descr + "'");
      c.e.push_back(x);
      c.v.push_back(y);
    }
    if (c.e.empty()) throw Error(name + ": no cross-section values after '" + descr + "'");
    out.push_back(std::move(c));
    k = j;
  }
}

// ------------------------------------------------------------------ request
struct StateProp {
  double energy = 0, weight = 1, population = 0;
  bool has_energy = false, has_weight = false, has_population = false;
};

struct Gas {
  std::string name;
  double mass = 0, fraction = 0, opb = -1;
  std::vector<Coll> colls;
};

}  // namespace

struct lgpu_request {
  lgpu_config cfg{};
  std::vector<lgpu_process> procs;
  std::vector<std::vector<double>> raw_e, raw_v;
  std::vector<lgpu_gas> gases;
  double emax_elastic = 0;
  std::vector<lgpu_conditions> jobs;
  // the collision behind each process for the EEDF post-processing, and its
  // tables (integral energies, values, momentum-transfer energies, values)
  std::vector<lgpu_twoterm_process> twoterm;
  std::vector<std::array<std::vector<double>, 4>> twoterm_tabs;
};

namespace {

// The momentum-transfer cross section a scattering law gives an integral one
// (Collision.C:127-199): sigma_m = sigma (1 - 2 pi Int_0^pi I cos sin dtheta),
// the integral by the trapezoidal rule over n_ang angles in [0, pi] laid out
// as Eigen's LinSpaced lays them; isotropic: sigma_m = sigma; forward: 0.
// I(e, theta) is the law's angular distribution, normalised so that
// 2 pi Int_0^pi I sin(theta) dtheta = 1 (AngularDistributionFunctions.h:32-110):
// Born dipole (Vialetto et al. 2021, eq. 23), Surendra (Vahedi and Surendra
// 1995, eq. 7), screened Coulomb (Hagelaar et al. 2000, eqs. 21-23); the
// momentum-conserving ionization law is 1/(4 pi). The factors that depend on
// the angle alone or on the energy alone are computed once; every term keeps
// the order of operations of the distributions, so it rounds the same.
std::vector<double> momentum_transfer(int law, const std::vector<double>& par, double thr, int n_ang,
                                      const std::vector<double>& e, const std::vector<double>& v) {
  if (law == 0) return v;
  if (law == 1) return std::vector<double>(v.size(), 0.0);
  if (n_ang < 2) throw Error("anisotropicScattering.angleNumber must be at least 2");
  const double iso = 1.0 / (4.0 * M_PI);
  const double step = M_PI / (n_ang - 1.0);
  std::vector<double> ang(n_ang), aux(n_ang), cs(n_ang), sh2(n_ang);
  for (int j = 0; j < n_ang; ++j) {
    ang[j] = j == n_ang - 1 ? M_PI : (double)j * step;
    aux[j] = std::cos(ang[j]) * std::sin(ang[j]);
    cs[j] = std::cos(ang[j]);
    const double sh = std::sin(ang[j] / 2.0);
    sh2[j] = sh * sh;  // pow(x, 2) rounds as x * x
  }
  std::vector<double> dist(n_ang);
  std::vector<double> m(v.size());
  for (size_t i = 0; i < e.size(); ++i) {
    const double en = e[i];
    if (law == 2) {  // Born dipole
      const double ea = en - thr;
      if (ea <= 0) {
        std::fill(dist.begin(), dist.end(), iso);
      } else {
        const double r = 2.0 * std::sqrt(en * ea), se = std::sqrt(en), sa = std::sqrt(ea);
        const double lg = std::log((sa + se) / std::sqrt(thr));
        for (int j = 0; j < n_ang; ++j) {
          const double q2 = ea + en - r * cs[j];
          dist[j] = 1.0 / (4.0 * M_PI) * se * sa / q2 / lg;
        }
      }
    } else if (law == 3) {  // Surendra
      if (en == 0) {
        std::fill(dist.begin(), dist.end(), iso);
      } else {
        const double lg = std::log(1.0 + en);
        for (int j = 0; j < n_ang; ++j) dist[j] = en / (4.0 * M_PI * (1.0 + en * sh2[j]) * lg);
      }
    } else if (law == 4) {  // screened Coulomb: the incident energy (p0 = 0) or the energy after the loss
      const double eps = (par.size() > 0 && par[0] != 0) ? en - thr : en;
      if (eps <= 0) {
        std::fill(dist.begin(), dist.end(), iso);
      } else {
        const double sp = (par.size() > 1 ? par[1] : 0.0) / eps;
        const double num = (sp * (sp + 1.0)) / M_PI, b = 2.0 * sp + 1.0;
        for (int j = 0; j < n_ang; ++j) {
          const double d = b - cs[j];
          dist[j] = num / (d * d);
        }
      }
    } else {
      std::fill(dist.begin(), dist.end(), iso);
    }
    double integ = aux[0] * dist[0];
    for (int j = 1; j < n_ang - 1; ++j) integ += 2.0 * aux[j] * dist[j];
    integ += aux[n_ang - 1] * dist[n_ang - 1];
    integ *= M_PI * step;
    m[i] = v[i] * (1.0 - integ);
  }
  return m;
}

// a state family "G(X,v=*)" matches "G(X,v=3)"
bool matches(const std::string& pattern, const std::string& name) {
  const size_t star = pattern.find('*');
  if (star == std::string::npos) return pattern == name;
  const std::string pre = pattern.substr(0, star), post = pattern.substr(star + 1);
  return name.size() >= pre.size() + post.size() && name.compare(0, pre.size(), pre) == 0 &&
         name.compare(name.size() - post.size(), post.size(), post) == 0 &&
         name.find(',', pre.size()) == std::string::npos;
}

// the hierarchy of a state: "G(X,v=0,J=2)" -> G(X), G(X,v=0), G(X,v=0,J=2)
std::vector<std::string> hierarchy(const std::string& state) {
  std::vector<std::string> out;
  const size_t open = state.find('('), close = state.rfind(')');
  if (open == std::string::npos || close == std::string::npos) return {state};
  const std::string base = state.substr(0, open);
  const auto levels = split_top(state.substr(open + 1, close - open - 1), ',');
  std::string acc;
  for (size_t k = 0; k < levels.size(); ++k) {
    acc += (k ? "," : "") + levels[k];
    out.push_back(base + "(" + acc + ")");
  }
  return out;
}

void parse_request(const std::string& setup, const std::map<std::string, std::string>& files, lgpu_request& r) {
  const auto root = read_setup(setup);
  const Node* wc = root->child("workingConditions");
  const Node* ek = root->child("electronKinetics");
  if (!wc || !ek) throw Error("the setup needs 'workingConditions' and 'electronKinetics'");
  if (!ek->child("eedfType") || ek->child("eedfType")->value != "boltzmannMC")
    throw Error("electronKinetics.eedfType must be boltzmannMC");
  auto num = [&](const Node* base, const char* key, double dflt) {
    const Node* n = base ? base->child(key) : nullptr;
    return (n && !n->value.empty()) ? value_of(n->value) : dflt;
  };
  // working conditions; one of them may be a vector (Setup.h:166-181)
  const double pressure = num(wc, "gasPressure", NAN), tg = num(wc, "gasTemperature", NAN);
  if (!(pressure > 0) || !(tg > 0)) throw Error("workingConditions needs gasPressure and gasTemperature");
  std::vector<double> en{0.0}, bn{0.0}, angle{180.0}, freq{0.0};
  const char* vec_key = nullptr;
  for (auto& kv : {std::make_pair("reducedElecField", &en), std::make_pair("reducedMagField", &bn),
                   std::make_pair("elecFieldAngle", &angle), std::make_pair("excitationFrequency", &freq)}) {
    const Node* n = wc->child(kv.first);
    if (!n) continue;
    *kv.second = values_of(n->value);
    if (kv.second->size() > 1) {
      if (vec_key) throw Error(std::string("only one working condition may be a vector: ") + vec_key + ", " + kv.first);
      vec_key = kv.first;
    }
  }
  const size_t n_jobs = std::max(std::max(en.size(), bn.size()), std::max(angle.size(), freq.size()));
  for (size_t k = 0; k < n_jobs; ++k) {
    lgpu_conditions c{};
    c.gas_density = pressure / (kBoltzmann * tg);
    c.gas_temperature = tg;
    c.reduced_field_td = en[std::min(k, en.size() - 1)];
    c.reduced_mag_field_hx = bn[std::min(k, bn.size() - 1)];
    c.field_angle_deg = angle[std::min(k, angle.size() - 1)];
    c.excitation_freq_hz = freq[std::min(k, freq.size() - 1)];
    r.jobs.push_back(c);
  }
  // numerics (BoltzmannMC.h:262-376); collision limits are multiples of nElectrons
  lgpu_config_default(&r.cfg);
  const Node* nm = ek->child("numericsMC");
  r.cfg.n_electrons = num(nm, "nElectrons", r.cfg.n_electrons);
  r.cfg.n_interp = (int)num(nm, "nInterpPoints", r.cfg.n_interp);
  r.cfg.init_temp_ratio = num(nm, "initialElecTempOverGasTemp", r.cfg.init_temp_ratio);
  r.cfg.min_coll_before_ss = num(nm, "minCollisionsBeforeSteadyState", r.cfg.min_coll_before_ss);
  r.cfg.max_coll_before_ss = num(nm, "maxCollisionsBeforeSteadyState", r.cfg.max_coll_before_ss);
  r.cfg.max_coll_after_ss = num(nm, "maxCollisionsAfterSteadyState", r.cfg.max_coll_after_ss);
  r.cfg.req_integration_points = num(nm, "nIntegrationPoints", r.cfg.req_integration_points);
  r.cfg.req_ss_times = num(nm, "nIntegratedSSTimes", r.cfg.req_ss_times);
  r.cfg.req_abs_time = num(nm, "integratedAbsoluteTime", r.cfg.req_abs_time);
  r.cfg.n_energy_cells = (int)num(nm, "nEnergyCells", r.cfg.n_energy_cells);
  r.cfg.n_cos_cells = (int)num(nm, "nCosAngleCells", r.cfg.n_cos_cells);
  r.cfg.n_radial_cells = (int)num(nm, "nRadialVelocityCells", r.cfg.n_radial_cells);
  r.cfg.n_axial_cells = (int)num(nm, "nAxialVelocityCells", r.cfg.n_axial_cells);
  r.cfg.n_phases = (int)num(nm, "nIntegrationPhases", r.cfg.n_phases);
  r.cfg.sync_x = num(nm, "synchronizationTimeXMaxCollisionFrequency", r.cfg.sync_x);
  r.cfg.sync_oversampling = (int)num(nm, "synchronizationOverSampling", r.cfg.sync_oversampling);
  r.cfg.seed = (uint64_t)num(nm, "gpuSeed", (double)r.cfg.seed);
  if (nm && nm->child("gasTemperatureEffect")) {
    const std::string g = nm->child("gasTemperatureEffect")->value;
    if (g == "true") r.cfg.gas_temperature_effect = 1;
    else if (g == "smartActivation") r.cfg.gas_temperature_effect = 2;
    else if (g == "false") r.cfg.gas_temperature_effect = 0;
    else throw Error("numericsMC.gasTemperatureEffect: '" + g + "'");
  }
  if (const Node* re = nm ? nm->child("relError") : nullptr) {
    r.cfg.errors_checked = 1;
    r.cfg.req_err_mean_energy = num(re, "meanEnergy", r.cfg.req_err_mean_energy);
    r.cfg.req_err_flux_v = num(re, "fluxDriftVelocity", r.cfg.req_err_flux_v);
    r.cfg.req_err_flux_d = num(re, "fluxDiffusionCoeffs", r.cfg.req_err_flux_d);
    r.cfg.req_err_bulk_v = num(re, "bulkDriftVelocity", r.cfg.req_err_bulk_v);
    r.cfg.req_err_bulk_d = num(re, "bulkDiffusionCoeffs", r.cfg.req_err_bulk_d);
    r.cfg.req_err_power = num(re, "powerBalance", r.cfg.req_err_power);
  }
  if (const Node* io = ek->child("ionizationOperatorType")) {
    const std::string s = io->value;
    if (s == "equalSharing") r.cfg.sharing = 0;
    else if (s == "oneTakesAll") r.cfg.sharing = 1;
    else if (s == "usingSDCS") r.cfg.sharing = 2;
    else if (s == "randomUniform") r.cfg.sharing = 3;
    else throw Error("ionizationOperatorType: '" + s + "'");
  }
  // collisions, gases in order of appearance
  std::vector<Coll> colls;
  const Node* lf = ek->child("LXCatFiles");
  if (!lf || lf->items.empty()) throw Error("electronKinetics.LXCatFiles lists no file");
  for (const std::string& f : lf->items) {
    auto it = files.find(f);
    if (it == files.end()) throw Error("the LXCat file '" + f + "' was not given");
    read_lxcat(f, it->second, colls);
  }
  std::vector<Gas> gases;
  for (Coll& c : colls) {
    const std::string g = gas_of(c.target);
    size_t k = 0;
    while (k < gases.size() && gases[k].name != g) ++k;
    if (k == gases.size()) {
      gases.push_back(Gas());
      gases.back().name = g;
    }
    gases[k].colls.push_back(c);
  }
  const Node* gp = ek->child("gasProperties");
  for (auto& kv : assignments(gp ? gp->child("mass") : nullptr))
    for (Gas& g : gases)
      if (g.name == kv.first) g.mass = value_of(kv.second);
  for (auto& kv : assignments(gp ? gp->child("fraction") : nullptr))
    for (Gas& g : gases)
      if (g.name == kv.first) g.fraction = value_of(kv.second);
  for (auto& kv : assignments(gp ? gp->child("OPBParameter") : nullptr))
    for (Gas& g : gases)
      if (g.name == kv.first) g.opb = value_of(kv.second);
  for (Gas& g : gases) {
    if (g.mass <= 0)
      for (const Coll& c : g.colls)
        if (c.type == "Elastic" && c.mass_ratio > 0) g.mass = kElectronMass / c.mass_ratio;
    if (g.mass <= 0) throw Error("no mass for the gas '" + g.name + "' (gasProperties.mass)");
  }
  // states: every state named by a collision, with the setup's properties
  std::map<std::string, StateProp> states;
  for (const Gas& g : gases)
    for (const Coll& c : g.colls)
      for (const std::string& s : {c.target, c.product})
        for (const std::string& h : hierarchy(s)) states[h];
  const Node* sp = ek->child("stateProperties");
  if (sp)
    for (const auto& ch : sp->children)
      if (ch.first != "energy" && ch.first != "statisticalWeight" && ch.first != "population")
        throw Error("stateProperties." + ch.first + " is not read by this front end");
  auto apply = [&](const char* key, int which) {
    for (auto& kv : assignments(sp ? sp->child(key) : nullptr)) {
      const size_t at = kv.second.find('@');
      if (at != std::string::npos) {
        if (which != 2 || kv.second.substr(0, at) != "boltzmannPopulation")
          throw Error(std::string("stateProperties.") + key + ": '" + kv.second + "' is not read by this front end");
        const std::string arg = trim(kv.second.substr(at + 1));
        const double t = arg == "gasTemperature" ? tg : value_of(arg);
        double z = 0;
        for (auto& st : states)
          if (matches(kv.first, st.first)) z += st.second.weight * std::exp(-st.second.energy * kElectronCharge / (kBoltzmann * t));
        for (auto& st : states)
          if (matches(kv.first, st.first)) {
            st.second.population =
                z > 0 ? st.second.weight * std::exp(-st.second.energy * kElectronCharge / (kBoltzmann * t)) / z : 0.0;
            st.second.has_population = true;
          }
        continue;
      }
      const double v = value_of(kv.second);
      for (auto& st : states) {
        if (!matches(kv.first, st.first)) continue;
        if (which == 0) st.second.energy = v, st.second.has_energy = true;
        else if (which == 1) st.second.weight = v, st.second.has_weight = true;
        else st.second.population = v, st.second.has_population = true;
      }
    }
  };
  apply("energy", 0);
  apply("statisticalWeight", 1);
  apply("population", 2);
  auto density = [&](const Gas& g, const std::string& state) {
    double d = g.fraction;
    for (const std::string& h : hierarchy(state)) d *= states[h].population;
    return d;
  };
  // angular scattering laws: "group;gas;type;law;params"
  std::map<std::pair<std::string, std::string>, std::pair<int, std::vector<double>>> laws;
  int n_angles = 0;
  const Node* an = ek->child("anisotropicScattering");
  if (an && an->child("isOn") && an->child("isOn")->value == "true") {
    if (an->child("angleNumber")) n_angles = (int)value_of(an->child("angleNumber")->value);
    const Node* lines = an->child("collisions");
    for (const std::string& it : lines ? lines->items : std::vector<std::string>()) {
      const auto f = split_top(no_spaces(it), ';');
      if (f.size() < 4 || f[0] != "group")
        throw Error("anisotropicScattering.collisions: only 'group;gas;type;law;params' lines are read: '" + it + "'");
      static const std::map<std::string, int> kLaw = {{"isotropic", 0}, {"forward", 1}, {"bornDipole", 2},
                                                      {"surendra", 3}, {"coulombScreen", 4},
                                                      {"momentumConservationIonization", 5}};
      auto lw = kLaw.find(f[3]);
      if (lw == kLaw.end()) throw Error("anisotropicScattering: unknown law '" + f[3] + "'");
      std::vector<double> p;
      if (f.size() > 4 && !f[4].empty())
        for (const std::string& t : split_top(f[4], ',')) p.push_back(value_of(t));
      laws[{f[1], f[2]}] = {lw->second, p};
    }
  }
  // flattening (BoltzmannMC.C:29-271)
  r.emax_elastic = 1e100;
  int it = 0;
  for (const Gas& g : gases) {
    lgpu_gas lg{};
    lg.first = it;
    lg.fraction = g.fraction;
    for (const Coll& c : g.colls) {
      if (c.type == "Effective") continue;
      auto law = laws.find({g.name, c.type});
      const int sampler = law == laws.end() ? 0 : law->second.first;
      const std::vector<double> sp_par = law == laws.end() ? std::vector<double>() : law->second.second;
      if (!c.integral && sampler != 0)
        throw Error("the momentum-transfer cross section of '" + g.name + " " + c.type +
                    "' needs an angular integration this front end does not do; give the integral one");
      std::vector<double> e = c.e, v = c.v;
      if ((c.type == "Elastic" || c.type == "Effective") && e[0] != 0) {  // Collision.C:40-43
        e.insert(e.begin(), 0.0);
        v.insert(v.begin(), v[0]);
      }
      // the collision's own tables, as the end-of-job routines read them
      std::array<std::vector<double>, 4> tabs{e, v, e, momentum_transfer(sampler, sp_par, c.threshold, n_angles, e, v)};
      size_t below = 0;  // BoltzmannMC.C:139-147
      while (below < e.size() && e[below] < c.threshold) ++below;
      e.erase(e.begin(), e.begin() + (long)below);
      v.erase(v.begin(), v.begin() + (long)below);
      if (e.empty() || e[0] != c.threshold) {
        e.insert(e.begin(), c.threshold);
        v.insert(v.begin(), 0.0);
      }
      lgpu_process q{};
      q.type = c.type == "Ionization" ? 1 : (c.type == "Attachment" ? 2 : 0);
      q.is_super = 0;
      q.is_elastic = c.type == "Elastic";
      q.sampler = sampler;
      q.sampler_p0 = sp_par.size() > 0 ? sp_par[0] : 0.0;
      q.sampler_p1 = sp_par.size() > 1 ? sp_par[1] : 0.0;
      q.emin = c.threshold;
      q.emax = e.back();
      q.rel_dens = density(g, c.target);
      q.mass = g.mass;
      q.eloss = c.threshold;
      q.wparam = c.type == "Ionization" ? (g.opb >= 0 ? g.opb : c.threshold) : 0.0;
      if (c.type == "Elastic") r.emax_elastic = std::min(r.emax_elastic, e.back());
      r.procs.push_back(q);
      r.raw_e.push_back(e);
      r.raw_v.push_back(v);
      lgpu_twoterm_process tt{};
      tt.kind = c.type == "Elastic" ? 0 : 1;
      tt.ion = q.type == 1 ? 1 : (q.type == 2 ? 2 : 0);
      tt.density = q.rel_dens;
      tt.threshold = c.threshold;
      tt.mass_ratio = kElectronMass / g.mass;
      r.twoterm.push_back(tt);
      r.twoterm_tabs.push_back(tabs);
      ++it;
      if (c.reverse) {
        const StateProp& st = states[c.target];
        const StateProp& sp2 = states[c.product];
        if (!st.has_weight || !sp2.has_weight)
          throw Error("the reversible collision " + c.target + " <-> " + c.product + " needs both statistical weights");
        r.twoterm.back().stat_ratio = st.weight / sp2.weight;
        lgpu_twoterm_process ts = r.twoterm.back();
        ts.kind = 2;
        ts.ion = 0;
        ts.density = density(g, c.product);
        r.twoterm.push_back(ts);
        r.twoterm_tabs.push_back(tabs);
        lgpu_process s = q;
        s.is_super = 1;
        s.is_elastic = 0;
        s.type = 0;
        s.superw = st.weight / sp2.weight;
        s.emin = 0.0;
        s.emax = q.emax - c.threshold;
        s.rel_dens = density(g, c.product);
        s.eloss = -c.threshold;
        s.wparam = 0.0;
        r.procs.push_back(s);
        r.raw_e.push_back(std::vector<double>());
        r.raw_v.push_back(std::vector<double>());
        ++it;
      }
    }
    lg.last = it - 1;
    if (lg.last >= lg.first) r.gases.push_back(lg);
  }
  if (r.procs.empty()) throw Error("no collisions in the LXCat files");
  for (size_t p = 0; p < r.procs.size(); ++p) {
    r.procs[p].raw_len = (int)r.raw_e[p].size();
    r.procs[p].raw_e = r.raw_e[p].empty() ? nullptr : r.raw_e[p].data();
    r.procs[p].raw_v = r.raw_v[p].empty() ? nullptr : r.raw_v[p].data();
    lgpu_twoterm_process& t = r.twoterm[p];
    const auto& tb = r.twoterm_tabs[p];
    t.n_int = (int)tb[0].size();
    t.n_mom = (int)tb[2].size();
    t.int_e = tb[0].data();
    t.int_v = tb[1].data();
    t.mom_e = tb[2].data();
    t.mom_v = tb[3].data();
  }
}

}  // namespace

extern "C" {

int lgpu_request_parse(const char* setup_text, int n_files, const char* const* file_names,
                       const char* const* file_texts, lgpu_request** out, char* err, size_t err_size) {
  if (err && err_size) err[0] = 0;
  if (!setup_text || !out || n_files < 0 || (n_files > 0 && (!file_names || !file_texts))) return LGPU_ERR_BAD_ARG;
  *out = nullptr;
  std::map<std::string, std::string> files;
  for (int k = 0; k < n_files; ++k) {
    if (!file_names[k] || !file_texts[k]) return LGPU_ERR_BAD_ARG;
    files[file_names[k]] = file_texts[k];
  }
  auto r = std::make_unique<lgpu_request>();
  try {
    parse_request(setup_text, files, *r);
  } catch (const std::exception& e) {
    if (err && err_size) std::snprintf(err, err_size, "%s", e.what());
    return LGPU_ERR_BAD_ARG;
  }
  *out = r.release();
  return LGPU_OK;
}

int lgpu_request_jobs(const lgpu_request* req) { return req ? (int)req->jobs.size() : 0; }

int lgpu_request_job(const lgpu_request* req, int k, lgpu_job* job) {
  if (!req || !job || k < 0 || k >= (int)req->jobs.size()) return LGPU_ERR_BAD_ARG;
  job->config = req->cfg;
  job->procs = req->procs.data();
  job->n_procs = (int)req->procs.size();
  job->gases = req->gases.data();
  job->n_gases = (int)req->gases.size();
  job->emax_elastic = req->emax_elastic;
  job->conditions = req->jobs[k];
  job->twoterm = req->twoterm.data();
  return LGPU_OK;
}

void lgpu_request_free(lgpu_request* req) { delete req; }

int lgpu_server_submit_request(lgpu_server* server, const lgpu_request* req, long long* job_ids, int max_ids) {
  if (!server || !req || !job_ids || max_ids < (int)req->jobs.size()) return LGPU_ERR_BAD_ARG;
  for (int k = 0; k < (int)req->jobs.size(); ++k) {
    lgpu_job job;
    lgpu_request_job(req, k, &job);
    if (int rc = lgpu_server_submit(server, &job, &job_ids[k])) return rc;
  }
  return LGPU_OK;
}

}  // extern "C"
