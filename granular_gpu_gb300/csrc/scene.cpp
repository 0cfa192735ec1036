// scene.cpp — scene-JSON reader and scene construction.
//
// loadSceneConfig (main.cu:123-167), readBoundaryParticlesFromFile
// (main.cu:169-188) and init_granular_system (main.cu:746-1173), restated
// with the same float arithmetic, so a scene file yields the same particle
// sets the reference hands to its constructor.  nlohmann_json is replaced by
// the small reader below.  Compile with -ffp-contract=off.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <random>
#include <sstream>
#include <sys/stat.h>

#include "scene.h"

namespace gg {

void set_error(const std::string& msg);

// ------------------------------------------------------------ JSON

namespace {

struct Parser {
  const std::string& s;
  size_t i = 0;
  std::string err;
  explicit Parser(const std::string& t) : s(t) {}
  void ws() {
    while (i < s.size() && (s[i] == ' ' || s[i] == '\n' || s[i] == '\r' || s[i] == '\t')) ++i;
  }
  bool fail(const char* m) {
    if (err.empty()) err = std::string(m) + " at offset " + std::to_string(i);
    return false;
  }
  bool lit(const char* w) {
    size_t n = strlen(w);
    if (s.compare(i, n, w) != 0) return false;
    i += n;
    return true;
  }
  bool string(std::string& out) {
    if (i >= s.size() || s[i] != '"') return fail("expected string");
    ++i;
    out.clear();
    while (i < s.size() && s[i] != '"') {
      char c = s[i++];
      if (c == '\\') {
        if (i >= s.size()) return fail("bad escape");
        char e = s[i++];
        switch (e) {
          case 'n': out += '\n'; break;
          case 't': out += '\t'; break;
          case 'r': out += '\r'; break;
          case 'b': out += '\b'; break;
          case 'f': out += '\f'; break;
          case 'u': {
            if (i + 4 > s.size()) return fail("bad unicode escape");
            unsigned cp = (unsigned)strtoul(s.substr(i, 4).c_str(), nullptr, 16);
            i += 4;
            if (cp < 0x80) out += (char)cp;
            else out += '?';
            break;
          }
          default: out += e;
        }
      } else {
        out += c;
      }
    }
    if (i >= s.size()) return fail("unterminated string");
    ++i;
    return true;
  }
  bool value(Json& v, int depth) {
    if (depth > 64) return fail("nesting too deep");
    ws();
    if (i >= s.size()) return fail("unexpected end");
    char c = s[i];
    if (c == '{') {
      ++i;
      v.kind = Json::Object;
      ws();
      if (i < s.size() && s[i] == '}') {
        ++i;
        return true;
      }
      while (true) {
        ws();
        std::string k;
        if (!string(k)) return false;
        ws();
        if (i >= s.size() || s[i] != ':') return fail("expected ':'");
        ++i;
        Json child;
        if (!value(child, depth + 1)) return false;
        v.obj[k] = std::move(child);
        ws();
        if (i < s.size() && s[i] == ',') {
          ++i;
          continue;
        }
        if (i < s.size() && s[i] == '}') {
          ++i;
          return true;
        }
        return fail("expected ',' or '}'");
      }
    }
    if (c == '[') {
      ++i;
      v.kind = Json::Array;
      ws();
      if (i < s.size() && s[i] == ']') {
        ++i;
        return true;
      }
      while (true) {
        Json child;
        if (!value(child, depth + 1)) return false;
        v.arr.push_back(std::move(child));
        ws();
        if (i < s.size() && s[i] == ',') {
          ++i;
          continue;
        }
        if (i < s.size() && s[i] == ']') {
          ++i;
          return true;
        }
        return fail("expected ',' or ']'");
      }
    }
    if (c == '"') {
      v.kind = Json::String;
      return string(v.str);
    }
    if (lit("true")) {
      v.kind = Json::Bool;
      v.b = true;
      return true;
    }
    if (lit("false")) {
      v.kind = Json::Bool;
      v.b = false;
      return true;
    }
    if (lit("null")) {
      v.kind = Json::Null;
      return true;
    }
    // number
    const char* start = s.c_str() + i;
    char* end = nullptr;
    double d = strtod(start, &end);
    if (end == start) return fail("unexpected character");
    i += (size_t)(end - start);
    v.kind = Json::Number;
    v.num = d;
    return true;
  }
};

}  // namespace

bool json_parse(const std::string& text, Json& out, std::string& err) {
  Parser p(text);
  if (!p.value(out, 0)) {
    err = p.err;
    return false;
  }
  p.ws();
  if (p.i != text.size()) {
    err = "trailing characters at offset " + std::to_string(p.i);
    return false;
  }
  return true;
}

// ------------------------------------------------------------ scene

namespace {

struct V3 {
  float x, y, z;
};
inline V3 v3(float x, float y, float z) { return V3{x, y, z}; }
inline V3 operator+(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline V3 operator-(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline V3 operator*(V3 a, V3 b) { return v3(a.x * b.x, a.y * b.y, a.z * b.z); }
inline V3 operator/(V3 a, V3 b) { return v3(a.x / b.x, a.y / b.y, a.z / b.z); }
inline V3 operator*(float s, V3 a) { return v3(s * a.x, s * a.y, s * a.z); }
inline V3 operator/(V3 a, float s) { return v3(a.x / s, a.y / s, a.z / s); }

struct SceneError {
  std::string msg;
};

double need_num(const Json& j, const char* k) {
  const Json* v = j.get(k);
  if (!v || v->kind != Json::Number) throw SceneError{std::string("scene key '") + k + "' missing or not a number"};
  return v->num;
}

V3 need_v3(const Json& j, const char* k) {
  const Json* v = j.get(k);
  if (!v || v->kind != Json::Object) throw SceneError{std::string("scene key '") + k + "' missing or not an object"};
  return v3((float)need_num(*v, "x"), (float)need_num(*v, "y"), (float)need_num(*v, "z"));
}

std::string opt_str(const Json& j, const char* k) {
  const Json* v = j.get(k);
  return (v && v->kind == Json::String) ? v->str : std::string();
}

bool file_exists(const std::string& p) {
  struct stat st;
  return !p.empty() && stat(p.c_str(), &st) == 0 && S_ISREG(st.st_mode);
}

// readBoundaryParticlesFromFile, main.cu:169-188: whitespace xyz triples.
std::vector<V3> read_points(const std::string& path) {
  std::vector<V3> pts;
  std::ifstream f(path);
  float x, y, z;
  while (f >> x >> y >> z) pts.push_back(v3(x, y, z));
  return pts;
}

void push(std::vector<float>& dst, V3 p) {
  dst.push_back(p.x);
  dst.push_back(p.y);
  dst.push_back(p.z);
}

}  // namespace

gg_status scene_build(const char* json_path, const char* base_dir, SceneData& out) {
  std::ifstream in(json_path);
  if (!in.is_open()) {
    set_error(std::string("Unable to open config file: ") + json_path);
    return GG_ERR_IO;
  }
  std::stringstream ss;
  ss << in.rdbuf();
  Json j;
  std::string err;
  if (!json_parse(ss.str(), j, err) || j.kind != Json::Object) {
    set_error(std::string("scene JSON parse error in ") + json_path + ": " + (err.empty() ? "not an object" : err));
    return GG_ERR_PARSE;
  }
  try {
    // loadSceneConfig, main.cu:123-167
    const V3 space = need_v3(j, "space_size");
    const float dt = (float)need_num(j, "dt");
    const V3 G = need_v3(j, "gravity");
    const V3 box = need_v3(j, "box_size");
    (void)need_num(j, "sph_spacing");
    const float init_spacing = (float)need_num(j, "init_spacing");
    (void)need_num(j, "smoothing_radius");
    const float cell_length = (float)need_num(j, "cell_length");
    const float density = (float)need_num(j, "density");
    const int scene = (int)need_num(j, "scene");
    const V3 btrans = need_v3(j, "boundary_translation");
    const V3 ptrans = need_v3(j, "particle_translation");
    const int is_adaptive = (int)need_num(j, "is_adaptive");
    const std::string obj_file = opt_str(j, "obj_file");
    out.save_file = opt_str(j, "save_file");
    if (!(cell_length > 0.0f)) throw SceneError{"cell_length must be positive"};
    const int cs[3] = {(int)std::ceil(space.x / cell_length), (int)std::ceil(space.y / cell_length),
                       (int)std::ceil(space.z / cell_length)};

    // granular lattice, main.cu:751-760 (x steps with j, y with i)
    out.particles.clear();
    for (int i = 0; (float)i < box.x; ++i)
      for (int jj = 0; (float)jj < box.y; ++jj)
        for (int k = 0; (float)k < box.z; ++k)
          push(out.particles, v3(0.27f + init_spacing * (float)jj, 0.13f + init_spacing * (float)i,
                                 0.17f + init_spacing * (float)k) +
                                  ptrans);
    const size_t np = out.particles.size() / 3;

    // 25 upsampled points per particle, main.cu:804-816.  The reference
    // passes three draws as arguments of make_float3, whose evaluation
    // order C++ leaves open; GCC (nvcc's host compiler) evaluates them right
    // to left, so z takes the first draw.
    {
      const float particle_radius = 0.01f;  // main.cu:46
      std::default_random_engine gen;
      std::uniform_real_distribution<float> dist(-particle_radius, particle_radius);
      out.upsampled.clear();
      out.upsampled.reserve(np * 25 * 3);
      for (size_t p = 0; p < np; ++p) {
        const V3 base = v3(out.particles[3 * p], out.particles[3 * p + 1], out.particles[3 * p + 2]);
        for (int n = 0; n < 25; ++n) {
          const float oz = dist(gen);
          const float oy = dist(gen);
          const float ox = dist(gen);
          push(out.upsampled, base + v3(ox, oy, oz));
        }
      }
    }

    // boundary walls, main.cu:822-1167
    std::vector<V3> pos;
    std::vector<int32_t> anim;
    const int c0 = 2 * cs[0], c1 = 2 * cs[1], c2 = 2 * cs[2];
    const V3 den = v3((float)(c0 - 1), (float)(c1 - 1), (float)(c2 - 1));
    auto wall = [&](int a, int b, int c) {
      const V3 x = v3((float)a, (float)b, (float)c) / den * space;
      pos.push_back(0.99f * x + 0.005f * space);
    };
    auto front_back = [&](bool back) {
      for (int i = 0; i < c0; ++i)
        for (int jj = 0; jj < c1; ++jj) {
          wall(i, jj, 0);
          if (back) wall(i, jj, c2 - 1);
        }
    };
    auto top_bottom = [&](bool top) {
      for (int i = 0; i < c0; ++i)
        for (int jj = 0; jj < c2 - 2; ++jj) {
          wall(i, 0, jj + 1);
          if (top) wall(i, c1 - 1, jj + 1);
        }
    };
    auto left_right = [&](bool right) {
      for (int i = 0; i < c1 - 2; ++i)
        for (int jj = 0; jj < c2 - 2; ++jj) {
          wall(0, i + 1, jj + 1);
          if (right) wall(c0 - 1, i + 1, jj + 1);
        }
    };
    auto translate = [&]() {
      for (auto& p : pos) p = p + btrans;
    };
    std::string obj_path = obj_file;
    if (!obj_file.empty() && base_dir && *base_dir) obj_path = std::string(base_dir) + "/" + obj_file;
    int is_move = 0;
    enum { PILING = 0, BOX = 1, EXCAVATOR = 2, FUNNEL = 3, CORNER = 4, BOX_OPENING = 5 };
    if (scene == PILING) {
      top_bottom(true);
      translate();
    } else if (scene == BOX || scene == BOX_OPENING) {
      front_back(true);
      top_bottom(true);
      left_right(true);
      translate();
    } else if (scene == EXCAVATOR) {
      front_back(true);
      top_bottom(false);
      left_right(true);
      anim.assign(pos.size(), 0);
      if (file_exists(obj_path)) {
        std::vector<V3> extra = read_points(obj_path);
        // the animation state (main.cu:940-951): the loaded range, and its
        // centroid before the bucket is placed
        gg_animation& A = out.animation;
        A.start_index = (int32_t)pos.size();
        A.num_particles = (int32_t)extra.size();
        A.is_animating = 1;
        A.animation_time = 0.0f;
        V3 centroid = v3(0.0f, 0.0f, 0.0f);
        for (const auto& p : extra) centroid = centroid + p;
        centroid = centroid / (float)extra.size();
        A.rotation_center[0] = centroid.x;
        A.rotation_center[1] = centroid.y;
        A.rotation_center[2] = centroid.z;
        for (auto& p : extra) p = p + v3(2.5f, 0.0f, 0.5f);
        anim.insert(anim.end(), extra.size(), 1);
        pos.insert(pos.end(), extra.begin(), extra.end());
      }
      is_move = 1;
    } else if (scene == FUNNEL) {
      front_back(true);
      top_bottom(false);
      left_right(true);
      anim.assign(pos.size(), 0);
      if (file_exists(obj_path)) {
        std::vector<V3> extra = read_points(obj_path);
        // the animation state (main.cu:1031-1034); the rotation centre keeps
        // its initialiser
        out.animation.start_index = (int32_t)pos.size();
        out.animation.num_particles = (int32_t)extra.size();
        out.animation.is_animating = 1;
        out.animation.animation_time = 0.0f;
        V3 centroid = v3(0.0f, 0.0f, 0.0f);
        for (const auto& p : extra) centroid = centroid + p;
        centroid = centroid / (float)extra.size();
        const float angle = (float)(90.0f * M_PI / 180.0f);
        const float cos_t = cosf(angle), sin_t = sinf(angle);
        for (auto& p : extra) {
          const V3 c = p - centroid;
          const float ny = c.y * cos_t - c.z * sin_t;
          const float nz = c.y * sin_t + c.z * cos_t;
          p = v3(c.x, ny, nz) + centroid + v3(1.25f, 0.3f, 1.5f);
        }
        anim.insert(anim.end(), extra.size(), 1);
        pos.insert(pos.end(), extra.begin(), extra.end());
      }
    } else if (scene == CORNER) {
      front_back(false);
      top_bottom(false);
      left_right(false);
      translate();
    }
    if (anim.size() < pos.size()) anim.resize(pos.size(), 0);
    out.boundary.clear();
    for (const auto& p : pos) push(out.boundary, p);
    out.animated = anim;

    // GranularSystem constructor arguments, main.cu:1169-1172
    gg_desc& d = out.desc;
    memset(&d, 0, sizeof(d));
    d.space_size[0] = space.x;
    d.space_size[1] = space.y;
    d.space_size[2] = space.z;
    d.cell_length = cell_length;
    d.dt = dt;
    d.gravity[0] = G.x;
    d.gravity[1] = G.y;
    d.gravity[2] = G.z;
    d.cell_size[0] = cs[0];
    d.cell_size[1] = cs[1];
    d.cell_size[2] = cs[2];
    d.density = density;
    d.upsampled_radius = 0.005f;  // main.cu:42
    d.is_move_boundary = is_move;
    d.is_adaptive = is_adaptive;
    gg_default_params(&d.params);
  } catch (const SceneError& e) {
    set_error(std::string(json_path) + ": " + e.msg);
    return GG_ERR_PARSE;
  }
  return GG_OK;
}

}  // namespace gg
