// config.cc - the data formats on either side of the render loop of
// main.cpp: the config.ini keys it reads (main.cpp:29-56, parsed with the
// vendored inipp) and the PPM P3 files it writes, including the progressive
// "bonus" snapshots and the side-by-side strip that main.cpp asks ImageMagick
// for (main.cpp:222-243).
#include <cstdio>
#include <cstring>
#include <fstream>
#include <map>
#include <sstream>
#include <string>

#include "../../include/tpt.h"

namespace {

// Whitespace as std::isspace in the "C" locale.
bool is_space(char c) { return c == ' ' || c == '\t' || c == '\n' || c == '\r' || c == '\f' || c == '\v'; }

std::string trim_left(const std::string &x) {
  size_t i = 0;
  while (i < x.size() && is_space(x[i])) i++;
  return x.substr(i);
}
std::string trim_right(const std::string &x) {
  size_t n = x.size();
  while (n > 0 && is_space(x[n - 1])) n--;
  return x.substr(0, n);
}

typedef std::map<std::string, std::map<std::string, std::string>> Sections;

// INI grammar of inipp::Ini::parse: lines are trimmed; ';' at the start is a
// comment; "[name]" opens a section; "key = value" (first '=', not at the
// start) adds a key to the current section unless it is already there (the
// first definition wins); everything else is ignored.
Sections parse_ini(const std::string &text) {
  Sections out;
  std::string section;
  std::istringstream is(text);
  std::string line;
  while (std::getline(is, line)) {
    line = trim_right(trim_left(line));
    if (line.empty() || line[0] == ';') continue;
    if (line[0] == '[') {
      if (line.back() == ']') section = line.substr(1, line.size() - 2);
      continue;
    }
    const size_t eq = line.find('=');
    if (eq == 0 || eq == std::string::npos) continue;
    const std::string key = trim_right(line.substr(0, eq));
    const std::string value = trim_left(line.substr(eq + 1));
    auto &sec = out[section];
    if (sec.find(key) == sec.end()) sec[key] = value;
  }
  return out;
}

// inipp::extract: the whole value must convert (trailing blanks allowed);
// otherwise the destination keeps its value.
template <class T>
void extract(const Sections &ini, const char *section, const char *key, T &dst) {
  auto s = ini.find(section);
  if (s == ini.end()) return;
  auto k = s->second.find(key);
  if (k == s->second.end()) return;
  std::istringstream is(k->second);
  T v;
  char c;
  if ((is >> std::boolalpha >> v) && !(is >> c)) dst = v;
}

}  // namespace

extern "C" {

void tpt_config_default(tpt_config *c) {  // main.cpp:31-40
  if (!c) return;
  c->width = 400;
  c->height = 200;
  c->sample = 10;
  c->recur_depth = 50;
  c->fov = 90.0f;
  c->allow_bonus_pic = 0;
  c->bonus_pic = 10;
  c->aperture = 0.2f;
  c->start_time = 0.0f;
  c->end_time = 1.0f;
}

tpt_status tpt_config_parse(const char *text, tpt_config *c) {  // main.cpp:42-56
  if (!text || !c) return TPT_ERR_INVALID_ARGUMENT;
  const Sections ini = parse_ini(text);
  int w = c->width, h = c->height, ns = c->sample, depth = c->recur_depth, allow = c->allow_bonus_pic,
      bonus = c->bonus_pic;
  float fov = c->fov, aperture = c->aperture, t0 = c->start_time, t1 = c->end_time;
  extract(ini, "DEFAULT", "width", w);
  extract(ini, "DEFAULT", "height", h);
  extract(ini, "DEFAULT", "sample", ns);
  extract(ini, "DEFAULT", "recur_depth", depth);
  extract(ini, "DEFAULT", "fov", fov);
  extract(ini, "DEFAULT", "bonus_pic", bonus);
  extract(ini, "DEFAULT", "allow_bonus_pic", allow);
  extract(ini, "BLUR", "aperture", aperture);
  extract(ini, "CAM_MOTION", "start_time", t0);
  extract(ini, "CAM_MOTION", "end_time", t1);
  c->width = w;
  c->height = h;
  c->sample = ns;
  c->recur_depth = depth;
  c->fov = fov;
  c->allow_bonus_pic = allow;
  c->bonus_pic = bonus;
  c->aperture = aperture;
  c->start_time = t0;
  c->end_time = t1;
  return TPT_OK;
}

tpt_status tpt_config_load(const char *path, tpt_config *c) {
  if (!path || !c) return TPT_ERR_INVALID_ARGUMENT;
  std::ifstream f(path);
  if (!f) return TPT_OK;  // main.cpp:29 never checks the stream: the defaults stand
  std::stringstream ss;
  ss << f.rdbuf();
  return tpt_config_parse(ss.str().c_str(), c);
}

tpt_status tpt_write_ppm_strip(const char *path, const uint8_t *const *images, int32_t count, int32_t w, int32_t h) {
  if (!path || !images || count <= 0 || w <= 0 || h <= 0) return TPT_ERR_INVALID_ARGUMENT;
  for (int k = 0; k < count; k++)
    if (!images[k]) return TPT_ERR_INVALID_ARGUMENT;
  FILE *f = std::fopen(path, "w");
  if (!f) return TPT_ERR_INVALID_ARGUMENT;
  std::fprintf(f, "P3\n%d %d\n255\n", w * count, h);
  for (int y = 0; y < h; y++)
    for (int k = 0; k < count; k++)
      for (int x = 0; x < w; x++) {
        const uint8_t *px = images[k] + 3 * ((size_t)y * w + x);
        std::fprintf(f, "%d %d %d \n", px[0], px[1], px[2]);
      }
  std::fclose(f);
  return TPT_OK;
}

// PPM reader for image textures (the reference decodes earthmap.jpg with
// stb_image, utils.cc:236-240; PPM is the decoder-free stand-in).
static bool ppm_token(FILE *f, std::string &tok) {
  tok.clear();
  int c = std::fgetc(f);
  for (;;) {
    while (c != EOF && is_space((char)c)) c = std::fgetc(f);
    if (c == '#') {  // comment to the end of the line
      while (c != EOF && c != '\n') c = std::fgetc(f);
      continue;
    }
    break;
  }
  while (c != EOF && !is_space((char)c) && c != '#') {
    tok.push_back((char)c);
    c = std::fgetc(f);
  }
  if (c == '#') std::ungetc(c, f);
  return !tok.empty();
}

static bool ppm_int(FILE *f, long &v) {
  std::string t;
  if (!ppm_token(f, t)) return false;
  char *end = nullptr;
  v = std::strtol(t.c_str(), &end, 10);
  return end && *end == 0 && v >= 0;
}

tpt_status tpt_read_ppm(const char *path, uint8_t *rgb8, int64_t cap, int32_t *w, int32_t *h) {
  if (!path || !w || !h || cap < 0 || (cap > 0 && !rgb8)) return TPT_ERR_INVALID_ARGUMENT;
  FILE *f = std::fopen(path, "rb");
  if (!f) return TPT_ERR_INVALID_ARGUMENT;
  std::string magic;
  long W = 0, H = 0, maxv = 0;
  tpt_status st = TPT_OK;
  if (!ppm_token(f, magic) || (magic != "P3" && magic != "P6") || !ppm_int(f, W) || !ppm_int(f, H) ||
      !ppm_int(f, maxv) || W <= 0 || H <= 0 || W > (1 << 16) || H > (1 << 16) || maxv <= 0 || maxv > 255) {
    st = TPT_ERR_PARSE;
  } else {
    *w = (int32_t)W;
    *h = (int32_t)H;
    const int64_t n = (int64_t)W * H * 3;
    if (rgb8 && cap >= n) {
      for (int64_t i = 0; i < n && st == TPT_OK; i++) {
        long v = 0;
        if (magic == "P3") {
          if (!ppm_int(f, v) || v > maxv) st = TPT_ERR_PARSE;
        } else {
          const int c = std::fgetc(f);
          if (c == EOF || c > maxv) st = TPT_ERR_PARSE;
          v = c;
        }
        rgb8[i] = (uint8_t)(maxv == 255 ? v : (v * 255 + maxv / 2) / maxv);
      }
    } else if (rgb8) {
      st = TPT_ERR_INVALID_ARGUMENT;  // buffer smaller than width*height*3
    }
  }
  std::fclose(f);
  return st;
}

}  // extern "C"
