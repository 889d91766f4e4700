#include "integrals.h"

#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstdio>
#include <fstream>
#include <numeric>
#include <sstream>
#include <stdexcept>

#include "dense.h"

namespace bgpu {

void Integrals::resize(int n) {
  norb = n;
  orbsym.assign(n, 0);
  t.assign((size_t)n * n, 0.0);
  v.assign((size_t)n * n * n * n, 0.0);
}

void Integrals::set_eri(int i, int j, int k, int l, double x) {
  const size_t n = norb;
  auto at = [&](int a, int b, int c, int d) -> double& { return v[((a * n + b) * n + c) * n + d]; };
  at(i, j, k, l) = x; at(j, i, k, l) = x; at(i, j, l, k) = x; at(j, i, l, k) = x;
  at(k, l, i, j) = x; at(l, k, i, j) = x; at(k, l, j, i) = x; at(l, k, j, i) = x;
}

static std::string upper(std::string s) {
  for (auto& c : s) c = (char)std::toupper((unsigned char)c);
  return s;
}

Integrals read_fcidump(const std::string& path) {
  std::ifstream f(path);
  if (!f) throw std::runtime_error("cannot open FCIDUMP: " + path);
  std::string header, line;
  while (std::getline(f, line)) {
    header += " " + line;
    std::string u = upper(line);
    if (u.find("&END") != std::string::npos || u.find("/") != std::string::npos) break;
  }
  // tokenise header on = , whitespace
  std::string h = upper(header);
  for (auto& c : h)
    if (c == ',' || c == '=' || c == '\t') c = ' ';
  std::istringstream hs(h);
  std::vector<std::string> tok;
  std::string w;
  while (hs >> w) tok.push_back(w);
  Integrals I;
  int norb = -1;
  std::vector<int> orbsym;
  for (size_t i = 0; i < tok.size(); ++i) {
    if (tok[i] == "NORB" && i + 1 < tok.size()) norb = std::stoi(tok[i + 1]);
    else if (tok[i] == "NELEC" && i + 1 < tok.size()) I.nelec = std::stoi(tok[i + 1]);
    else if (tok[i] == "MS2" && i + 1 < tok.size()) I.ms2 = std::stoi(tok[i + 1]);
    else if (tok[i] == "ISYM" && i + 1 < tok.size()) I.isym = std::stoi(tok[i + 1]) - 1;
    else if (tok[i] == "ORBSYM") {
      size_t k = i + 1;
      while (k < tok.size() && std::isdigit((unsigned char)tok[k][0])) orbsym.push_back(std::stoi(tok[k++]) - 1);
    }
  }
  if (norb <= 0) throw std::runtime_error("FCIDUMP header without NORB: " + path);
  I.resize(norb);
  for (int i = 0; i < norb && i < (int)orbsym.size(); ++i) I.orbsym[i] = orbsym[i];
  // value i j k l per line (1-based; k = l = 0: one-electron; all 0: core
  // energy), input.C:1421-1663; Fortran D exponents are accepted, anything
  // else that is not five numbers with indices in 0..norb is an error
  long lineno = 0;
  while (std::getline(f, line)) {
    ++lineno;
    std::istringstream ls(line);
    std::vector<std::string> t;
    while (ls >> w) t.push_back(w);
    if (t.empty() || t[0][0] == '!') continue;  // blank and comment lines (ReadMeaningfulLine)
    auto bad = [&](const char* why) {
      return std::runtime_error(std::string("FCIDUMP ") + path + ": " + why + " in integral line " +
                                std::to_string(lineno) + ": " + line);
    };
    if (t.size() != 5) throw bad("expected value i j k l");
    for (auto& c : t[0])
      if (c == 'D' || c == 'd') c = 'E';
    double x;
    int idx[4];
    try {
      size_t used = 0;
      x = std::stod(t[0], &used);
      if (used != t[0].size()) throw std::invalid_argument("value");
      for (int q = 0; q < 4; ++q) {
        idx[q] = std::stoi(t[q + 1], &used);
        if (used != t[q + 1].size()) throw std::invalid_argument("index");
      }
    } catch (const std::logic_error&) {
      throw bad("unreadable number");
    }
    for (int q = 0; q < 4; ++q)
      if (idx[q] < 0 || idx[q] > norb) throw bad("orbital index out of range");
    const int i = idx[0], j = idx[1], k = idx[2], l = idx[3];
    if (i == 0 && j == 0 && k == 0 && l == 0) I.ecore = x;
    else if (k == 0 && l == 0) {
      if (i == 0 || j == 0) throw bad("one-electron integral with orbital 0");
      I.t[(size_t)(i - 1) * norb + (j - 1)] = x;
      I.t[(size_t)(j - 1) * norb + (i - 1)] = x;
    } else {
      if (i == 0 || j == 0 || k == 0 || l == 0) throw bad("two-electron integral with orbital 0");
      I.set_eri(i - 1, j - 1, k - 1, l - 1, x);
    }
  }
  return I;
}

void write_fcidump(const Integrals& I, const std::string& path) {
  FILE* f = std::fopen(path.c_str(), "w");
  if (!f) throw std::runtime_error("cannot write " + path);
  std::fprintf(f, " &FCI NORB=%d,NELEC=%d,MS2=%d,\n  ORBSYM=", I.norb, I.nelec, I.ms2);
  for (int p = 0; p < I.norb; ++p) std::fprintf(f, "%d,", I.orbsym[p] + 1);
  std::fprintf(f, "\n  ISYM=%d\n &END\n", I.isym + 1);
  const int n = I.norb;
  for (int p = 0; p < n; ++p)
    for (int q = 0; q <= p; ++q)
      for (int r = 0; r < n; ++r)
        for (int s = 0; s <= r; ++s) {
          if (p * (p + 1) / 2 + q < r * (r + 1) / 2 + s) continue;
          const double x = I.g(p, q, r, s);
          if (x != 0.0) std::fprintf(f, "%23.16e %4d %4d %4d %4d\n", x, p + 1, q + 1, r + 1, s + 1);
        }
  for (int p = 0; p < n; ++p)
    for (int q = 0; q <= p; ++q)
      if (I.h(p, q) != 0.0) std::fprintf(f, "%23.16e %4d %4d %4d %4d\n", I.h(p, q), p + 1, q + 1, 0, 0);
  std::fprintf(f, "%23.16e %4d %4d %4d %4d\n", I.ecore, 0, 0, 0, 0);
  std::fclose(f);
}

Integrals reorder(const Integrals& I, const std::vector<int>& perm) {
  Integrals O = I;
  const int n = I.norb;
  O.order.resize(n);
  for (int a = 0; a < n; ++a) O.order[a] = I.order.empty() ? perm[a] : I.order[perm[a]];
  for (int a = 0; a < n; ++a) {
    O.orbsym[a] = I.orbsym[perm[a]];
    for (int b = 0; b < n; ++b) O.t[(size_t)a * n + b] = I.h(perm[a], perm[b]);
  }
  for (int a = 0; a < n; ++a)
    for (int b = 0; b < n; ++b)
      for (int c = 0; c < n; ++c)
        for (int d = 0; d < n; ++d)
          O.v[(((size_t)a * n + b) * n + c) * n + d] = I.g(perm[a], perm[b], perm[c], perm[d]);
  return O;
}

std::vector<int> fiedler_order(const Integrals& I) {
  const int n = I.norb;
  std::vector<double> K((size_t)n * n, 0.0);
  // FCIDUMP lists each unique integral once; (ij|ij) with i>=j is the entry
  // read for the exchange graph, and 1e-7 |h_ij| is added
  for (int i = 0; i < n; ++i)
    for (int j = 0; j <= i; ++j) {
      const double kij = std::fabs(I.g(i, j, i, j)) + 1.0e-7 * std::fabs(I.h(i, j));
      K[(size_t)i * n + j] = K[(size_t)j * n + i] = kij;
    }
  std::vector<double> lap((size_t)n * n, 0.0);
  for (int i = 0; i < n; ++i) {
    double rs = 0.0;
    for (int j = 0; j < n; ++j) rs += K[(size_t)i * n + j];
    for (int j = 0; j < n; ++j) lap[(size_t)i * n + j] = -K[(size_t)i * n + j];
    lap[(size_t)i * n + i] += rs;
  }
  std::vector<double> w(n), V((size_t)n * n);
  jacobi_eigh(n, lap.data(), w.data(), V.data());
  std::vector<double> f(n);
  for (int i = 0; i < n; ++i) f[i] = V[(size_t)i * n + (n > 1 ? 1 : 0)];
  std::vector<int> idx(n);
  std::iota(idx.begin(), idx.end(), 0);
  std::stable_sort(idx.begin(), idx.end(), [&](int a, int b) { return f[a] < f[b]; });
  return idx;
}

std::vector<int> orbital_order(const Integrals& I, const std::string& how) {
  std::vector<int> perm(I.norb);
  std::iota(perm.begin(), perm.end(), 0);
  if (how == "noreorder") return perm;
  if (how == "fiedler") return fiedler_order(I);
  if (how.rfind("file:", 0) == 0) {
    std::ifstream f(how.substr(5));
    if (!f) throw std::runtime_error("cannot open reorder file " + how.substr(5));
    perm.clear();
    std::string tok;
    while (f >> tok) {
      for (auto& c : tok)
        if (c == ',') c = ' ';
      std::istringstream ts(tok);
      int x;
      while (ts >> x) perm.push_back(x - 1);
    }
    if ((int)perm.size() != I.norb) throw std::runtime_error("reorder file has wrong length");
    return perm;
  }
  throw std::runtime_error("unknown reorder option " + how);
}

uint64_t Rng::next() {
  uint64_t z = (s += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

double Rng::uniform() { return ((next() >> 11) + 0.5) * (1.0 / 9007199254740992.0); }

double Rng::normal() {
  const double u1 = uniform(), u2 = uniform();
  return std::sqrt(-2.0 * std::log(u1)) * std::cos(2.0 * 3.14159265358979323846 * u2);
}

Integrals synthetic_hamiltonian(int n, int nelec, int nchol, uint64_t seed, bool d2h, double dlo, double dhi,
                                double hsd, double lsd) {
  Integrals I;
  I.resize(n);
  I.nelec = nelec;
  I.ms2 = 0;
  I.isym = 0;
  for (int p = 0; p < n; ++p) I.orbsym[p] = d2h ? (p % 8) : 0;
  Rng rng(seed);
  for (int p = 0; p < n; ++p) {
    I.t[(size_t)p * n + p] = (n > 1) ? dlo + (dhi - dlo) * p / (n - 1) : dlo;
    for (int q = 0; q < p; ++q) {
      const double x = hsd * rng.normal();
      I.t[(size_t)p * n + q] = I.t[(size_t)q * n + p] = x;
    }
  }
  std::vector<double> L((size_t)nchol * n * n);
  for (int k = 0; k < nchol; ++k)
    for (int p = 0; p < n; ++p)
      for (int q = 0; q <= p; ++q) {
        const double x = lsd * rng.normal();
        L[((size_t)k * n + p) * n + q] = L[((size_t)k * n + q) * n + p] = x;
      }
  // (pq|rs) = sum_k L^k_pq L^k_rs  as a symmetric n^2 x n^2 product
  const size_t n2 = (size_t)n * n;
  for (size_t a = 0; a < n2; ++a)
    for (size_t b = 0; b <= a; ++b) {
      double s = 0.0;
      for (int k = 0; k < nchol; ++k) s += L[(size_t)k * n2 + a] * L[(size_t)k * n2 + b];
      I.v[a * n2 + b] = I.v[b * n2 + a] = s;
    }
  if (d2h) {
    for (int p = 0; p < n; ++p)
      for (int q = 0; q < n; ++q)
        if (I.orbsym[p] != I.orbsym[q]) I.t[(size_t)p * n + q] = 0.0;
    for (int p = 0; p < n; ++p)
      for (int q = 0; q < n; ++q)
        for (int r = 0; r < n; ++r)
          for (int s = 0; s < n; ++s)
            if ((I.orbsym[p] ^ I.orbsym[q] ^ I.orbsym[r] ^ I.orbsym[s]) != 0)
              I.v[(((size_t)p * n + q) * n + r) * n + s] = 0.0;
  }
  return I;
}

const ScheduleEntry& Config::entry(int sweep) const {
  const ScheduleEntry* e = &schedule.front();
  for (auto& s : schedule)
    if (s.iter <= sweep) e = &s;
  return *e;
}

static std::vector<std::string> split_ws(const std::string& s) {
  std::istringstream is(s);
  std::vector<std::string> v;
  std::string w;
  while (is >> w) v.push_back(w);
  return v;
}

static std::string lower(std::string s) {
  for (auto& c : s) c = (char)std::tolower((unsigned char)c);
  return s;
}

Config parse_config_text(const std::string& text, const std::string& base_dir) {
  Config c;
  std::istringstream in(text);
  std::string line;
  bool sweep_tol_set = false;
  auto next_meaningful = [&](std::string& out) -> bool {
    while (std::getline(in, out)) {
      auto p = out.find_first_of("!#");
      if (p != std::string::npos) out = out.substr(0, p);
      if (!split_ws(out).empty()) return true;
    }
    return false;
  };
  while (next_meaningful(line)) {
    auto tok = split_ws(line);
    const std::string key = lower(tok[0]);
    auto need = [&](size_t k) {
      if (tok.size() <= k) throw std::runtime_error("dmrg.conf: keyword " + key + " needs a value");
    };
    if (key == "nelec") { need(1); c.nelec = std::stoi(tok[1]); }
    else if (key == "spin") { need(1); c.spin = std::stoi(tok[1]); }
    else if (key == "irrep") { need(1); c.irrep = std::stoi(tok[1]) - 1; }
    else if (key == "sym") { need(1); c.sym = lower(tok[1]); }
    else if (key == "orbitals") {
      need(1);
      c.orbitals = tok[1];
      if (!c.orbitals.empty() && c.orbitals[0] != '/' && !base_dir.empty()) c.orbitals = base_dir + "/" + c.orbitals;
    } else if (key == "maxiter") { need(1); c.maxiter = std::stoi(tok[1]); }
    else if (key == "sweep_tol" || key == "sweep_tolerance") {
      need(1);
      sweep_tol_set = true;
      const std::string v = lower(tok[1]);
      if (v == "loose") c.sweep_tol = 1e-4;
      else if (v == "tight") c.sweep_tol = 1e-7;
      else if (v == "verytight") c.sweep_tol = 1e-9;
      else c.sweep_tol = std::stod(tok[1]);
    } else if (key == "nroots") { need(1); c.nroots = std::stoi(tok[1]); }
    else if (key == "weights") {
      c.weights.clear();
      for (size_t i = 1; i < tok.size(); ++i) c.weights.push_back(std::stod(tok[i]));
    } else if (key == "noreorder" || key == "nofiedler") c.reorder = "noreorder";
    else if (key == "fiedler") c.reorder = "fiedler";
    else if (key == "reorder") {
      need(1);
      std::string p = tok[1];
      if (p[0] != '/' && !base_dir.empty()) p = base_dir + "/" + p;
      c.reorder = "file:" + p;
    } else if (key == "outputlevel") { need(1); c.outputlevel = std::stoi(tok[1]); }
    else if (key == "startm") { need(1); c.startM = std::stoi(tok[1]); }
    else if (key == "maxm") { need(1); c.maxM = std::stoi(tok[1]); }
    else if (key == "seed") { need(1); c.seed = std::stoull(tok[1]); }
    else if (key == "deflation_max_size" || key == "max_deflation_size") { need(1); c.deflation_max = std::stoi(tok[1]); }
    else if (key == "deflation_min_size") { need(1); c.deflation_min = std::stoi(tok[1]); }
    else if (key == "davidson_max_iter") {
      need(1);
      c.davidson_max_iter = std::stoi(tok[1]);
      if (c.davidson_max_iter < 1) throw std::runtime_error("davidson_max_iter must be positive");
    }
    else if (key == "warmup") { if (tok.size() > 1) c.warmup = lower(tok[1]); }
    else if (key == "restart" || key == "fullrestart") c.restart = true;
    else if (key == "spill") c.spill = true;
    else if (key == "onepdm" || key == "onerdm" || key == "ordm") c.onepdm = true;
    else if (key == "tran_onepdm") c.onepdm = c.tran_onepdm = true;
    else if (key == "prefix" || key == "scratch") {
      need(1);
      std::string p = tok[1];
      if (p[0] != '/' && !base_dir.empty()) p = base_dir + "/" + p;
      c.prefix = p;
    }
    else if (key == "reset_iter" || key == "reset_iters" || key == "reset_iterations") c.reset_iter = true;
    else if (key == "checkpoint") {
      need(1);
      std::string p = tok[1];
      if (p[0] != '/' && !base_dir.empty()) p = base_dir + "/" + p;
      c.checkpoint = p;
    }
    else if (key == "hubbard" || key == "heisenberg" || key == "nonspinadapted" || key == "bcs" || key == "onedot")
      throw std::runtime_error("dmrg.conf keyword not supported on this path: " + key);
    else if (key == "schedule") {
      if (tok.size() > 1 && lower(tok[1]) == "default") {
        c.schedule_default = true;
        continue;
      }
      c.schedule.clear();
      std::string sl;
      while (next_meaningful(sl)) {
        auto st = split_ws(sl);
        if (lower(st[0]) == "end") break;
        if (st.size() != 4) throw std::runtime_error("schedule lines need 4 entries: " + sl);
        ScheduleEntry e;
        e.iter = std::stoi(st[0]);
        e.M = std::stoi(st[1]);
        e.davidson_tol = std::stod(st[2]);
        e.noise = std::stod(st[3]);
        c.schedule.push_back(e);
      }
    }
    else if (key == "twodot_noise") {
      if (tok.size() != 3) throw std::runtime_error("twodot_noise needs two numbers (amplitude, gamma)");
      c.twodot_noise = std::stod(tok[1]);
    }
    // other keywords (hf_occ, twodot, twodot_to_onedot, twopdm, ...) are accepted and ignored
  }
  if (!sweep_tol_set && c.sweep_tol <= 0) c.sweep_tol = 1e-5;
  if (c.nroots > 1) {
    c.deflation_min = std::max(c.deflation_min, c.nroots);
    c.deflation_max = std::max(c.deflation_max, c.nroots + 20);
  }
  if (c.weights.empty()) c.weights.assign(c.nroots, 1.0 / c.nroots);
  if (c.restart && c.checkpoint.empty())
    c.checkpoint = (base_dir.empty() ? std::string(".") : base_dir) + "/bgpu_checkpoint.bin";
  if (c.schedule_default) make_default_schedule(c);
  if (c.schedule.empty()) throw std::runtime_error("dmrg.conf: no schedule");
  if (c.maxiter < c.schedule.back().iter) c.maxiter = c.schedule.back().iter + 2;
  return c;
}

Config parse_config(const std::string& path) {
  std::ifstream f(path);
  if (!f) throw std::runtime_error("cannot open " + path);
  std::stringstream ss;
  ss << f.rdbuf();
  std::string dir;
  auto p = path.find_last_of('/');
  if (p != std::string::npos) dir = path.substr(0, p);
  return parse_config_text(ss.str(), dir);
}

Integrals load_integrals(Config& c) {
  Integrals I0;
  const std::string key = "synthetic:";
  std::string o = c.orbitals;
  const auto pos = o.find(key);
  if (pos != std::string::npos) {
    std::string spec = o.substr(pos + key.size());
    for (auto& ch : spec)
      if (ch == ':') ch = ' ';
    std::istringstream is(spec);
    int norb = 0, nelec = 0, nchol = 0, d2h = 0;
    unsigned long long seed = 0;
    is >> norb >> nelec >> nchol >> seed >> d2h;
    if (norb <= 0) throw std::runtime_error("bad synthetic spec " + o);
    I0 = synthetic_hamiltonian(norb, nelec, nchol, seed, d2h != 0);
    if (d2h) c.sym = "d2h";
  } else {
    I0 = read_fcidump(o);
  }
  if (c.nelec < 0) c.nelec = I0.nelec;
  return reorder(I0, orbital_order(I0, c.reorder));
}

void make_default_schedule(Config& c) {
  // the reference's ladder (Schedule.C:13-98): M steps and sweeps per step
  const int defM[] = {50, 100, 250, 500, 1000, 2000, 3000, 4000, 5000, 6000, 7000, 8000, 9000, 10000};
  const int defIter[] = {8, 8, 8, 8, 8, 4, 4, 4, 4, 4, 4, 4, 4, 4};
  const double defTol[] = {1e-5, 1e-5, 1e-5, 1e-5, 5e-5, 5e-6, 5e-6, 5e-6, 5e-6, 5e-6, 5e-6, 5e-6, 5e-6, 5e-6};
  // scheduled (perturbative) noise; none when twodot_noise is given
  const double nz = c.twodot_noise > 0.0 ? 0.0 : 1.0;
  const double defNoise[] = {1e-4, 1e-4, 1e-4, 1e-4, 5e-5, 5e-5, 5e-5, 5e-5, 5e-5, 5e-5, 5e-5, 5e-5, 5e-5, 5e-5};
  if (c.maxM <= 0) throw std::runtime_error("schedule default needs maxM");
  c.schedule.clear();
  int count = 0;
  bool first = false;
  for (int i = 0; i < 14; ++i) {
    if (!first) {
      if (c.startM == c.maxM) {
        c.schedule.push_back({count, c.startM, 1e-5, nz * 1e-4});
        count += 8;
        c.schedule.push_back({count, c.startM, 5e-6, nz * 5e-5});
        break;
      } else if (c.startM == defM[i]) {
        first = true;
        c.schedule.push_back({count, defM[i], defTol[i], nz * defNoise[i]});
        count += defIter[i];
      } else if (c.startM < defM[i]) {
        first = true;
        const int j = i > 0 ? i - 1 : 0;
        c.schedule.push_back({count, c.startM, defTol[j], nz * defNoise[j]});
        count += defIter[j];
        c.schedule.push_back({count, defM[i], defTol[i], nz * defNoise[i]});
        count += defIter[i];
      }
    } else {
      if (defM[i] >= c.maxM) {
        c.schedule.push_back({count, c.maxM, defTol[i], nz * defNoise[i]});
        count += defIter[i];
        break;
      }
      c.schedule.push_back({count, defM[i], defTol[i], nz * defNoise[i]});
      count += defIter[i];
    }
  }
  const int last = c.schedule.back().iter;
  c.schedule.push_back({last + 2, c.maxM, c.sweep_tol / 10.0, 0.0});
  if (c.maxiter <= c.schedule.back().iter) c.maxiter = last + 6;
}

}  // namespace bgpu
