// Option parsing with the reference's names and semantics (no Boost).
#include "params.h"

#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <sstream>

namespace simrecon {

namespace {

enum Kind { kInt, kFloat, kShort, kUnsigned, kString, kSwitch, kBoolValue, kFloatList, kAngleList };

struct Opt {
  Kind kind;
  void* (*field)(Options*);
  // value a bare option (no '=value') stores; null for options that require one
  const char* implicit;
};

#define F(expr) [](Options* o) -> void* { return (void*)&(expr); }

const std::map<std::string, Opt>& table()
{
  // setupProgramOptions, cudaSirecon.cpp:917-1004
  static const std::map<std::string, Opt> t = {
      {"input-file", {kString, F(o->p.ifiles), nullptr}},
      {"output-file", {kString, F(o->p.ofiles), nullptr}},
      {"otf-file", {kString, F(o->p.otffiles), nullptr}},
      {"config", {kString, F(o->config_file), nullptr}},
      {"ndirs", {kInt, F(o->p.ndirs), nullptr}},
      {"nphases", {kInt, F(o->p.nphases), nullptr}},
      {"nordersout", {kInt, F(o->p.norders_output), nullptr}},
      {"angle0", {kFloat, F(o->p.k0startangle), nullptr}},
      {"ls", {kFloat, F(o->p.linespacing), nullptr}},
      {"na", {kFloat, F(o->p.na), nullptr}},
      {"nimm", {kFloat, F(o->p.nimm), nullptr}},
      {"wiener", {kFloat, F(o->p.wiener), nullptr}},
      {"otfcutoff", {kFloat, F(o->p.otfcutoff), nullptr}},
      {"zoomfact", {kFloat, F(o->p.zoomfact), nullptr}},
      {"zzoom", {kInt, F(o->p.z_zoom), nullptr}},
      {"background", {kFloat, F(o->p.constbkgd), nullptr}},
      {"usecorr", {kString, F(o->p.corrfiles), nullptr}},
      {"forcemodamp", {kFloatList, F(o->p.forceamp), nullptr}},
      {"k0angles", {kAngleList, F(o->p.k0angles), nullptr}},
      {"otfRA", {kSwitch, F(o->p.bRadAvgOTF), "1"}},
      {"otfPerAngle", {kSwitch, F(o->p.bOneOTFperAngle), "1"}},
      {"fastSI", {kSwitch, F(o->p.bFastSIM), "1"}},
      {"k0searchAll", {kInt, F(o->p.bUseTime0k0), "0"}},
      {"norescale", {kInt, F(o->p.do_rescale), "0"}},
      {"equalizez", {kSwitch, F(o->p.equalizez), "1"}},
      {"equalizet", {kSwitch, F(o->p.equalizet), "1"}},
      {"dampenOrder0", {kSwitch, F(o->p.bDampenOrder0), "1"}},
      {"nosuppress", {kInt, F(o->p.bSuppress_singularities), "0"}},
      {"nokz0", {kSwitch, F(o->p.bNoKz0), "1"}},
      {"gammaApo", {kFloat, F(o->p.apoGamma), nullptr}},
      {"explodefact", {kFloat, F(o->p.explodefact), nullptr}},
      {"nofilterovlps", {kBoolValue, F(o->p.bFilteroverlaps), "0"}},
      {"saveprefiltered", {kString, F(o->p.fileSeparated), nullptr}},
      {"savealignedraw", {kString, F(o->p.fileRawAligned), nullptr}},
      {"saveoverlaps", {kString, F(o->p.fileOverlaps), nullptr}},
      {"2lenses", {kSwitch, F(o->p.bTwolens), "1"}},
      {"bessel", {kSwitch, F(o->p.bBessel), "1"}},
      {"besselExWave", {kFloat, F(o->p.BesselLambdaEx), nullptr}},
      {"besselNA", {kFloat, F(o->p.BesselNA), nullptr}},
      {"deskew", {kFloat, F(o->p.deskewAngle), nullptr}},
      {"deskewshift", {kInt, F(o->p.extraShift), nullptr}},
      {"noRecon", {kSwitch, F(o->p.bNoRecon), "1"}},
      {"cropXY", {kUnsigned, F(o->p.cropXYto), nullptr}},
      {"xyres", {kFloat, F(o->ip.dxy), nullptr}},
      {"zres", {kFloat, F(o->ip.dz), nullptr}},
      {"zresPSF", {kFloat, F(o->p.dzPSF), nullptr}},
      {"wavelength", {kShort, F(o->ip.wave[0]), nullptr}},
      {"writeTitle", {kSwitch, F(o->p.bWriteTitle), "1"}},
      // extension: use the declared bool flags instead of the reference's
      // int-sized reads (default on = reference behaviour)
      {"referenceFlagBytes", {kSwitch, F(o->reference_flag_bytes), "1"}},
      // extension: the reference sets bBgInExtHdr only through ReconParams
      // (no option); per-section backgrounds from the MRC extended header
      {"bgInExtHdr", {kInt, F(o->p.bBgInExtHdr), "1"}},
  };
  return t;
}
#undef F

std::string trim(const std::string& s)
{
  size_t a = s.find_first_not_of(" \t\r\n");
  size_t b = s.find_last_not_of(" \t\r\n");
  return a == std::string::npos ? std::string() : s.substr(a, b - a + 1);
}

bool to_bool(const std::string& v, bool* out)
{
  std::string s;
  for (char c : v) s += (char)tolower((unsigned char)c);
  if (s.empty() || s == "1" || s == "true" || s == "yes" || s == "on") *out = true;
  else if (s == "0" || s == "false" || s == "no" || s == "off") *out = false;
  else return false;
  return true;
}

bool to_int(const std::string& v, long* out)
{
  char* end = nullptr;
  long x = strtol(v.c_str(), &end, 10);
  if (v.empty() || *end != '\0') return false;
  *out = x;
  return true;
}

bool to_float(const std::string& v, float* out)
{
  char* end = nullptr;
  float x = strtof(v.c_str(), &end);
  if (v.empty() || *end != '\0') return false;
  *out = x;
  return true;
}

}  // namespace

void set_defaults(Options* o)
{
  ReconParams& p = o->p;
  ImageParams& ip = o->ip;
  // SetDefaultParams (cudaSirecon.cpp:16-72) ...
  p.k0startangle = 1.57193f;
  p.linespacing = 0.177f;
  p.na = 1.36f;
  p.nimm = 1.515f;
  p.ndirs = 3;
  p.nphases = 3;
  p.phaseSteps = nullptr;
  p.norders_output = 0;
  p.norders = 0;
  p.bTwolens = false;
  p.bFastSIM = false;
  p.bBessel = false;
  p.BesselNA = 0.45f;
  p.otfcutoff = 0.006f;
  p.zoomfact = 2;
  p.z_zoom = 1;
  p.nzPadTo = 0;
  p.explodefact = 1.0f;
  p.bFilteroverlaps = true;
  p.recalcarrays = 1;
  p.napodize = 10;
  p.forceamp.assign(1, 0.f);
  p.bSearchforvector = 1;
  p.bUseTime0k0 = 1;
  p.apodizeoutput = 0;
  p.bSuppress_singularities = 1;
  p.suppression_radius = 10;
  p.bDampenOrder0 = false;
  p.bFitallphases = 1;
  p.do_rescale = 1;
  p.equalizez = false;
  p.equalizet = false;
  p.bNoKz0 = false;
  p.bRadAvgOTF = false;
  p.bOneOTFperAngle = false;
  p.bFixdrift = 0;
  p.drift_filter_fact = 0.0f;
  p.constbkgd = 0.0f;
  p.bBgInExtHdr = 0;
  p.bUsecorr = 0;
  p.electrons_per_bit = 0.6528f;
  p.readoutNoiseVar = 32.42f;
  p.bMakemodel = 0;
  p.bSaveAlignedRaw = 0;
  p.bSaveSeparated = 0;
  p.bSaveOverlaps = 0;
  p.bWriteTitle = false;
  p.bTIFF = false;
  p.wienerInr = 0.f;
  p.nxotf = p.nyotf = p.nzotf = 0;
  p.dkzotf = p.dkrotf = 0.f;
  // ... overridden by the program_options defaults (cudaSirecon.cpp:917-1004),
  // which notify() always writes
  p.ndirs = 3;
  p.nphases = 5;
  p.norders_output = 0;
  p.k0startangle = 1.648f;
  p.linespacing = 0.172f;
  p.na = 1.2f;
  p.nimm = 1.33f;
  p.wiener = 0.01f;
  p.otfcutoff = 0.006f;
  p.zoomfact = 2.f;
  p.z_zoom = 1;
  p.constbkgd = 0.f;
  p.bRadAvgOTF = false;
  p.bOneOTFperAngle = false;
  p.bFastSIM = false;
  p.equalizez = false;
  p.equalizet = false;
  p.bDampenOrder0 = false;
  p.bNoKz0 = false;
  p.apoGamma = 1.f;
  p.explodefact = 1.f;
  p.bTwolens = false;
  p.bBessel = false;
  p.BesselLambdaEx = 0.488f;
  p.BesselNA = 0.144f;
  p.deskewAngle = 0.f;
  p.extraShift = 0;
  p.bNoRecon = false;
  p.cropXYto = 0;
  p.dzPSF = 0.15f;
  p.bWriteTitle = false;
  ip = ImageParams{};
  ip.dxy = 0.1f;
  ip.dz = 0.2f;
  ip.wave[0] = 530;
  ip.ntimes = 1;
  ip.curTimeIdx = 0;
  ip.nwaves = 1;
  // gammaApo always has a value, so setParams sets apodizeoutput = 2
  // (cudaSirecon.cpp:1040-1045)
  p.apodizeoutput = 2;
  o->config_file.clear();
  o->help = o->version = false;
  o->reference_flag_bytes = true;
  o->given.clear();
}

bool apply_option(Options* o, const std::string& key, const std::string& value, bool has_value, std::string* err)
{
  if (key == "help" || key == "h") {
    o->help = true;
    return true;
  }
  if (key == "version") {
    o->version = true;
    return true;
  }
  std::string k = (key == "c") ? "config" : key;
  auto it = table().find(k);
  if (it == table().end()) {
    if (err) *err = "unrecognised option '" + key + "'";
    return false;
  }
  const Opt& op = it->second;
  std::string v = has_value ? trim(value) : std::string(op.implicit ? op.implicit : "");
  if (!has_value && !op.implicit) {
    if (err) *err = "option '" + key + "' requires a value";
    return false;
  }
  void* f = op.field(o);
  bool ok = true;
  switch (op.kind) {
    case kInt: {
      long x;
      ok = to_int(v, &x);
      if (ok) *(int*)f = (int)x;
      break;
    }
    case kUnsigned: {
      long x;
      ok = to_int(v, &x) && x >= 0;
      if (ok) *(unsigned*)f = (unsigned)x;
      break;
    }
    case kShort: {
      long x;
      ok = to_int(v, &x);
      if (ok) *(short*)f = (short)x;
      break;
    }
    case kFloat: {
      float x;
      ok = to_float(v, &x);
      if (ok) *(float*)f = x;
      break;
    }
    case kString: *(std::string*)f = v; break;
    case kSwitch:
    case kBoolValue: {
      bool b;
      ok = to_bool(v, &b);
      if (ok) *(bool*)f = b;
      break;
    }
    case kFloatList: {
      // multitoken: values separated by blanks (one per token on the CLI)
      std::vector<float>* vec = (std::vector<float>*)f;
      if (!o->given.count(k)) vec->clear();
      std::istringstream ss(v);
      std::string tok;
      while (ss >> tok) {
        float x;
        if (!to_float(tok, &x)) {
          ok = false;
          break;
        }
        vec->push_back(x);
      }
      break;
    }
    case kAngleList: {
      // comma-separated, converted with strtod (cudaSirecon.cpp:1062-1067)
      std::vector<float>* vec = (std::vector<float>*)f;
      vec->clear();
      std::stringstream ss(v);
      std::string tok;
      while (std::getline(ss, tok, ','))
        if (!tok.empty()) vec->push_back((float)strtod(tok.c_str(), nullptr));
      break;
    }
  }
  if (!ok) {
    if (err) *err = "invalid value '" + v + "' for option '" + key + "'";
    return false;
  }
  // setParams side effects (cudaSirecon.cpp:1011-1070)
  if (k == "usecorr") o->p.bUsecorr = 1;
  if (k == "saveprefiltered") o->p.bSaveSeparated = 1;
  if (k == "savealignedraw") o->p.bSaveAlignedRaw = 1;
  if (k == "saveoverlaps") o->p.bSaveOverlaps = 1;
  o->given.insert(k);
  return true;
}

bool apply_config_text(Options* o, const std::string& text, std::string* err)
{
  std::set<std::string> from_cli = o->given;
  std::istringstream in(text);
  std::string line;
  int lineno = 0;
  while (std::getline(in, line)) {
    ++lineno;
    size_t hash = line.find('#');
    if (hash != std::string::npos) line = line.substr(0, hash);
    line = trim(line);
    if (line.empty() || line[0] == '[') continue;
    size_t eq = line.find('=');
    if (eq == std::string::npos) {
      if (err) *err = "config line " + std::to_string(lineno) + ": expected key=value";
      return false;
    }
    std::string k = trim(line.substr(0, eq)), v = trim(line.substr(eq + 1));
    std::string kk = (k == "c") ? "config" : k;
    if (from_cli.count(kk)) continue;  // command-line values win
    if (!apply_option(o, k, v, true, err)) {
      if (err) *err = "config line " + std::to_string(lineno) + ": " + *err;
      return false;
    }
  }
  return true;
}

bool apply_config_file(Options* o, const std::string& path, bool must_exist, std::string* err)
{
  std::ifstream f(path);
  if (!f) {
    if (must_exist) {
      if (err) *err = "can not open config file: " + path;
      return false;
    }
    return true;
  }
  std::stringstream ss;
  ss << f.rdbuf();
  return apply_config_text(o, ss.str(), err);
}

bool parse_command_line(Options* o, int argc, char** argv, std::string* err)
{
  static const char* positional[] = {"input-file", "output-file", "otf-file"};
  int npos = 0;
  for (int i = 1; i < argc; ++i) {
    std::string a = argv[i] ? argv[i] : "";
    if (a.size() > 1 && a[0] == '-' && !(a.size() > 1 && (isdigit((unsigned char)a[1]) || a[1] == '.'))) {
      std::string body = a[1] == '-' ? a.substr(2) : a.substr(1);
      std::string key = body, val;
      bool has = false;
      size_t eq = body.find('=');
      if (eq != std::string::npos) {
        key = body.substr(0, eq);
        val = body.substr(eq + 1);
        has = true;
      }
      std::string k = (key == "c") ? "config" : key;
      auto it = table().find(k);
      bool needs_value = it != table().end() && it->second.implicit == nullptr;
      if (!has && needs_value) {
        if (i + 1 >= argc) {
          if (err) *err = "option '" + key + "' requires a value";
          return false;
        }
        val = argv[++i];
        has = true;
        // multitoken forcemodamp: swallow following numeric tokens
        if (k == "forcemodamp")
          while (i + 1 < argc && argv[i + 1][0] != '-') val += std::string(" ") + argv[++i];
      }
      if (!apply_option(o, key, val, has, err)) return false;
    } else {
      if (npos >= 3) {
        if (err) *err = "too many positional arguments";
        return false;
      }
      if (!apply_option(o, positional[npos++], a, true, err)) return false;
    }
  }
  if (o->help || o->version) return true;
  if (!o->config_file.empty()) {
    std::string e2;
    std::ifstream f(o->config_file);
    if (f && !apply_config_file(o, o->config_file, true, err)) return false;
  }
  if (o->p.otffiles.empty()) {
    if (err) *err = "the option '--otf-file' is required but missing";
    return false;
  }
  return true;
}

std::string usage_text()
{
  std::string s =
      "Usage:\n cudasirecon [--options] [option-arguments] input_file(or folder) output_file(or file name pattern) "
      "otf_file\n\n List of options:\n";
  for (const auto& kv : table()) s += "  --" + kv.first + "\n";
  s += "  -c [ --config ] arg\n  -h [ --help ]\n  --version\n";
  return s;
}

bool effective_nokz0(const Options& o)
{
  if (!o.reference_flag_bytes) return o.p.bNoKz0;
  // bytes 142..145 of ReconParams: bNoKz0, a padding byte (value-initialised
  // here, so zero) and the two low bytes of wiener (little-endian)
  uint32_t bits;
  memcpy(&bits, &o.p.wiener, 4);
  return o.p.bNoKz0 || (bits & 0xFFFFu) != 0;
}

}  // namespace simrecon
