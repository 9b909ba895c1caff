// emc.conf reader: the keys of configs.cpp:40-90 (read through libconfig by
// the reference) in the subset of libconfig syntax that emc.conf uses:
//   name = value;   or   name : value;   ('=' / ':' and ';' / ',' accepted,
//   the terminator optional at end of file)
//   values: integers (decimal or 0x hex), floats (with exponent), booleans
//   true/false (any case), "strings" (adjacent literals concatenate);
//   comments: '#' and '//' to end of line, '/* ... */'.
// Unknown keys are ignored (libconfig lookups ignore them too).  Keys the
// reference reads but emc.conf does not set (nGPU, blur_image, blur_sigma,
// exclude_ratio, model_blur) are left uninitialised by the reference; here
// they get the defaults of emc_config_defaults.  The reference's diff_type
// comparison tests "poisson" twice (configs.cpp:78-82), so "relative" never
// maps; here it maps to EMC_DIFF_RELATIVE.
#include <cctype>
#include <cerrno>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>

#include "../../../include/emc_gb300.h"

namespace {

struct Value {
  enum Kind { INT, FLOAT, BOOL, STRING } kind;
  long long i = 0;
  double f = 0.0;
  bool b = false;
  std::string s;
};

struct Parser {
  const std::string& t;
  size_t p = 0;
  int line = 1;
  std::string err;
  explicit Parser(const std::string& text) : t(text) {}

  void skip() {
    for (;;) {
      while (p < t.size() && std::isspace((unsigned char)t[p])) {
        if (t[p] == '\n') ++line;
        ++p;
      }
      if (p < t.size() && (t[p] == '#' || (t[p] == '/' && p + 1 < t.size() && t[p + 1] == '/'))) {
        while (p < t.size() && t[p] != '\n') ++p;
        continue;
      }
      if (p + 1 < t.size() && t[p] == '/' && t[p + 1] == '*') {
        p += 2;
        while (p + 1 < t.size() && !(t[p] == '*' && t[p + 1] == '/')) {
          if (t[p] == '\n') ++line;
          ++p;
        }
        p = p + 2 <= t.size() ? p + 2 : t.size();
        continue;
      }
      return;
    }
  }

  bool fail(const char* fmt, ...) {
    char buf[256];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    err = "line " + std::to_string(line) + ": " + buf;
    return false;
  }

  bool name(std::string& out) {
    skip();
    if (p >= t.size() || !(std::isalpha((unsigned char)t[p]) || t[p] == '*'))
      return fail("expected a setting name");
    size_t b = p;
    while (p < t.size() && (std::isalnum((unsigned char)t[p]) || t[p] == '_' || t[p] == '-' ||
                            t[p] == '*'))
      ++p;
    out = t.substr(b, p - b);
    return true;
  }

  bool value(Value& v) {
    skip();
    if (p >= t.size()) return fail("missing value");
    if (t[p] == '"') {
      v.kind = Value::STRING;
      v.s.clear();
      while (p < t.size() && t[p] == '"') {
        ++p;
        while (p < t.size() && t[p] != '"') {
          if (t[p] == '\\' && p + 1 < t.size()) {
            ++p;
            const char c = t[p];
            v.s += c == 'n' ? '\n' : c == 't' ? '\t' : c;
          } else {
            v.s += t[p];
          }
          ++p;
        }
        if (p >= t.size()) return fail("unterminated string");
        ++p;
        skip();
      }
      return true;
    }
    size_t b = p;
    while (p < t.size() && !std::isspace((unsigned char)t[p]) && t[p] != ';' && t[p] != ',' &&
           t[p] != '#')
      ++p;
    std::string tok = t.substr(b, p - b);
    std::string low = tok;
    for (auto& c : low) c = (char)std::tolower((unsigned char)c);
    if (low == "true" || low == "false") {
      v.kind = Value::BOOL;
      v.b = low == "true";
      return true;
    }
    char* end = nullptr;
    errno = 0;
    if (tok.find_first_of(".eE") != std::string::npos && low.rfind("0x", 0) != 0) {
      v.kind = Value::FLOAT;
      v.f = std::strtod(tok.c_str(), &end);
    } else {
      v.kind = Value::INT;
      v.i = std::strtoll(tok.c_str(), &end, 0);
      if (end && *end == 'L') ++end;
    }
    if (tok.empty() || !end || *end != '\0' || errno) return fail("bad value '%s'", tok.c_str());
    return true;
  }
};

bool as_int(const Value& v, int* out) {
  if (v.kind == Value::INT) *out = (int)v.i;
  else if (v.kind == Value::BOOL) *out = v.b ? 1 : 0;
  else if (v.kind == Value::FLOAT) *out = (int)v.f;
  else return false;
  return true;
}

bool as_double(const Value& v, double* out) {
  if (v.kind == Value::FLOAT) *out = v.f;
  else if (v.kind == Value::INT) *out = (double)v.i;
  else return false;
  return true;
}

void copy_str(char* dst, const std::string& s) {
  std::snprintf(dst, EMC_CONFIG_PATH_MAX, "%s", s.c_str());
}

}  // namespace

extern "C" int emc_config_defaults(emc_config* c) {
  if (!c) return EMC_ERR_INVALID;
  std::memset(c, 0, sizeof(*c));
  // emc.conf values (emc.conf:1-26) as the defaults of a missing key
  c->model_side = 64;
  c->read_stride = 4;
  c->wavelength = 1.03e-9;
  c->pixel_size = 75.0e-6;
  c->detector_size = 1024;
  c->detector_distance = 740.0e-3;
  c->rotations_n = 12;
  c->sigma_start = 0.4;
  c->sigma_final = 0.12;
  c->sigma_half_life = 25;
  c->diff = EMC_DIFF_POISSON;
  c->slice_chunk = 5000;
  c->N_images = 200;
  c->max_iterations = 1;
  c->normalize_images = 1;
  c->known_intensity = 0;
  c->model_input = 0;
  c->output_period = 1;
  c->isOutput = 1;
  c->nGPUs = 1;
  return EMC_OK;
}

extern "C" int emc_config_parse(const char* text, emc_config* c, char* err, int errlen) {
  if (!text || !c) return EMC_ERR_INVALID;
  std::string t(text);
  Parser ps(t);
  auto bad = [&](const std::string& m) {
    if (err && errlen > 0) std::snprintf(err, (size_t)errlen, "%s", m.c_str());
    return EMC_ERR_INVALID;
  };
  for (;;) {
    ps.skip();
    if (ps.p >= t.size()) break;
    std::string key;
    if (!ps.name(key)) return bad(ps.err);
    ps.skip();
    if (ps.p >= t.size() || (t[ps.p] != '=' && t[ps.p] != ':'))
      return bad("line " + std::to_string(ps.line) + ": expected '=' after " + key);
    ++ps.p;
    Value v;
    if (!ps.value(v)) return bad(ps.err);
    ps.skip();
    if (ps.p < t.size() && (t[ps.p] == ';' || t[ps.p] == ',')) ++ps.p;
    bool ok = true;
    const std::string& k = key;
    if (k == "model_side") ok = as_int(v, &c->model_side);
    else if (k == "read_stride") ok = as_int(v, &c->read_stride);
    else if (k == "wavelength") ok = as_double(v, &c->wavelength);
    else if (k == "pixel_size") ok = as_double(v, &c->pixel_size);
    else if (k == "detector_size") ok = as_int(v, &c->detector_size);
    else if (k == "detector_distance") ok = as_double(v, &c->detector_distance);
    else if (k == "rotations_n") ok = as_int(v, &c->rotations_n);
    else if (k == "sigma_start") ok = as_double(v, &c->sigma_start);
    else if (k == "sigma_final") ok = as_double(v, &c->sigma_final);
    else if (k == "sigma_half_life") ok = as_int(v, &c->sigma_half_life);
    else if (k == "slice_chunk") ok = as_int(v, &c->slice_chunk);
    else if (k == "N_images") ok = as_int(v, &c->N_images);
    else if (k == "max_iterations") ok = as_int(v, &c->max_iterations);
    else if (k == "blur_image") ok = as_int(v, &c->blur_image);
    else if (k == "blur_sigma") ok = as_double(v, &c->blur_sigma);
    else if (k == "normalize_images") ok = as_int(v, &c->normalize_images);
    else if (k == "known_intensity") ok = as_int(v, &c->known_intensity);
    else if (k == "model_input") ok = as_int(v, &c->model_input);
    else if (k == "exclude_images") ok = as_int(v, &c->exclude_images);
    else if (k == "exclude_ratio") ok = as_double(v, &c->exclude_ratio);
    else if (k == "model_blur") ok = as_double(v, &c->model_blur);
    else if (k == "isDebug") ok = as_int(v, &c->isDebug);
    else if (k == "isOutput") ok = as_int(v, &c->isOutput);
    else if (k == "output_loop") ok = as_int(v, &c->output_loop);
    else if (k == "output_period") ok = as_int(v, &c->output_period);
    else if (k == "nGPU") ok = as_int(v, &c->nGPUs);
    else if (k == "mask_file" || k == "image_prefix" || k == "model_file") {
      if (v.kind != Value::STRING) ok = false;
      else copy_str(k == "mask_file" ? c->mask_file : k == "image_prefix" ? c->image_prefix
                                                                          : c->model_file, v.s);
    } else if (k == "diff_type") {
      if (v.kind != Value::STRING) ok = false;
      else if (v.s == "absolute") c->diff = EMC_DIFF_ABSOLUTE;
      else if (v.s == "poisson") c->diff = EMC_DIFF_POISSON;
      else if (v.s == "relative") c->diff = EMC_DIFF_RELATIVE;
      else if (v.s == "true_poisson") c->diff = EMC_DIFF_TRUE_POISSON;
      else return bad("diff_type \"" + v.s + "\" is not absolute, poisson or relative");
    }
    if (!ok) return bad("line " + std::to_string(ps.line) + ": wrong type for " + k);
  }
  if (c->model_side <= 1 || c->N_images <= 0 || c->rotations_n <= 0 || c->slice_chunk <= 0 ||
      c->sigma_half_life <= 0)
    return bad("model_side, N_images, rotations_n, slice_chunk and sigma_half_life must be > 0");
  return EMC_OK;
}

extern "C" int emc_config_read(const char* path, emc_config* c, char* err, int errlen) {
  if (!path || !c) return EMC_ERR_INVALID;
  std::ifstream f(path);
  if (!f) {
    if (err && errlen > 0) std::snprintf(err, (size_t)errlen, "cannot open %s", path);
    return EMC_ERR_INVALID;
  }
  std::stringstream ss;
  ss << f.rdbuf();
  emc_config_defaults(c);
  return emc_config_parse(ss.str().c_str(), c, err, errlen);
}
