// writers.cpp — the reference's on-disk outputs of a frame (main.cu:190-694):
// ASCII VTK point clouds of the render points, of the particles split by
// mass and of the animated walls, the render-point CSV and the frame-time
// list.  The data come through gg_read; the formatting (default stream
// output of floats, points written "x z y") and the centring arithmetic
// (float sums in point order) are the reference's.
#include <cmath>
#include <filesystem>
#include <fstream>
#include <string>
#include <vector>

#include "gg_internal.h"

namespace {

struct F3 {
  float x, y, z;
};

gg_status read_pos(gg_system* S, gg_set set, std::vector<F3>& out) {
  int64_t n = 0;
  gg_status rc = gg_read(S, set, GG_FIELD_POS, nullptr, 0, &n);
  if (rc != GG_OK) return rc;
  out.resize((size_t)n);
  return n ? gg_read(S, set, GG_FIELD_POS, out.data(), n, &n) : GG_OK;
}

template <typename T>
gg_status read_field(gg_system* S, gg_set set, gg_field f, std::vector<T>& out) {
  int64_t n = 0;
  gg_status rc = gg_read(S, set, f, nullptr, 0, &n);
  if (rc != GG_OK) return rc;
  out.resize((size_t)n);
  return n ? gg_read(S, set, f, out.data(), n, &n) : GG_OK;
}

bool valid(const F3& p) { return !std::isnan(p.x) && !std::isnan(p.y) && !std::isnan(p.z); }

std::vector<F3> valid_only(const std::vector<F3>& pts) {
  std::vector<F3> v;
  v.reserve(pts.size());
  for (const F3& p : pts)
    if (valid(p)) v.push_back(p);
  return v;
}

// The reference's centring (main.cu:286-309, 482-497, 634-647): the centroid
// summed in point order in float and divided by the count, then the lowest
// centred y lifted to zero.
struct Centring {
  F3 c;
  float y_offset;
  F3 apply(const F3& p) const { return {p.x - c.x, p.y - c.y + y_offset, p.z - c.z}; }
};

Centring centring_of(const std::vector<F3>& pts, bool divide_when_empty) {
  F3 c{0.0f, 0.0f, 0.0f};
  for (const F3& p : pts) {
    c.x += p.x;
    c.y += p.y;
    c.z += p.z;
  }
  if (!pts.empty() || divide_when_empty) {
    const float k = (float)pts.size();
    c = {c.x / k, c.y / k, c.z / k};
  }
  float min_y = 1000000.f;
  for (const F3& p : pts) min_y = fminf(min_y, p.y - c.y);
  return {c, min_y < 0.0f ? -min_y : 0.0f};
}

bool write_points(std::ofstream& out, const char* title, const std::vector<F3>& pts) {
  out << "# vtk DataFile Version 3.0\n";
  out << title << "\n";
  out << "ASCII\n";
  out << "DATASET UNSTRUCTURED_GRID\n";
  out << "POINTS " << pts.size() << " float\n";
  for (const F3& p : pts) out << p.x << " " << p.z << " " << p.y << "\n";
  out << "CELLS " << pts.size() << " " << pts.size() * 2 << "\n";
  for (size_t i = 0; i < pts.size(); ++i) out << "1 " << i << "\n";
  out << "CELL_TYPES " << pts.size() << "\n";
  for (size_t i = 0; i < pts.size(); ++i) out << "1\n";
  return out.good();
}

gg_status open_out(const std::string& path, std::ofstream& out) {
  out.open(path);
  if (!out.is_open()) {
    gg::set_error("cannot open " + path);
    return GG_ERR_IO;
  }
  return GG_OK;
}

gg_status finish(std::ofstream& out, bool ok, const std::string& path) {
  out.close();
  if (!ok || out.fail()) {
    gg::set_error("write failed for " + path);
    return GG_ERR_IO;
  }
  return GG_OK;
}

// Animated wall particles (is_animated == 1), in wall order.
gg_status animated_walls(gg_system* S, std::vector<F3>& out) {
  std::vector<F3> b;
  std::vector<int32_t> anim;
  gg_status rc = read_pos(S, GG_SET_BOUNDARY, b);
  if (rc == GG_OK) rc = read_field(S, GG_SET_BOUNDARY, GG_FIELD_IS_ANIMATED, anim);
  if (rc != GG_OK) return rc;
  out.clear();
  for (size_t i = 0; i < b.size(); ++i)
    if (anim[i] == 1) out.push_back(b[i]);
  return GG_OK;
}

}  // namespace

extern "C" {

// saveUpsampledPositionsToVTK (main.cu:588-664): the set's valid points,
// centred.  The file is created even when no point is valid (then empty).
gg_status gg_write_vtk_centered(gg_system* S, gg_set set, const char* path) {
  if (!S || !path) {
    gg::set_error("gg_write_vtk_centered: null argument");
    return GG_ERR_INVALID_ARGUMENT;
  }
  std::vector<F3> pos;
  gg_status rc = read_pos(S, set, pos);
  if (rc != GG_OK) return rc;
  std::ofstream out;
  if ((rc = open_out(path, out)) != GG_OK) return rc;
  const std::vector<F3> v = valid_only(pos);
  if (v.empty()) return finish(out, true, path);
  const Centring t = centring_of(v, true);
  std::vector<F3> c;
  c.reserve(v.size());
  for (const F3& p : v) c.push_back(t.apply(p));
  return finish(out, write_points(out, "Upsampled Granular Particles", c), path);
}

// saveParticlesByMass (main.cu:256-368): the particles' valid points, centred,
// into <base>_mass_light (mass < 2), <base>_mass_medium (2 <= mass <= 3) and
// <base>_mass_heavy (the rest), one <frame_id>.vtk per non-empty group.
gg_status gg_write_vtk_by_mass(gg_system* S, const char* base, int32_t frame_id) {
  if (!S || !base) {
    gg::set_error("gg_write_vtk_by_mass: null argument");
    return GG_ERR_INVALID_ARGUMENT;
  }
  const std::string dirs[3] = {std::string(base) + "_mass_light", std::string(base) + "_mass_medium",
                               std::string(base) + "_mass_heavy"};
  std::error_code ec;
  for (const std::string& d : dirs) std::filesystem::create_directories(d, ec);
  std::vector<F3> pos;
  std::vector<float> mass;
  gg_status rc = read_pos(S, GG_SET_GRANULAR, pos);
  if (rc == GG_OK) rc = read_field(S, GG_SET_GRANULAR, GG_FIELD_MASS, mass);
  if (rc != GG_OK) return rc;
  const Centring t = centring_of(valid_only(pos), false);
  std::vector<F3> group[3];
  for (size_t i = 0; i < pos.size(); ++i) {
    if (!valid(pos[i])) continue;
    const F3 c = t.apply(pos[i]);
    const float m = mass[i];
    group[m < 2.0f ? 0 : (m >= 2.0f && m <= 3.0f ? 1 : 2)].push_back(c);
  }
  for (int g = 0; g < 3; ++g) {
    if (group[g].empty()) continue;
    const std::string path = dirs[g] + "/" + std::to_string(frame_id) + ".vtk";
    std::ofstream out;
    if ((rc = open_out(path, out)) != GG_OK) return rc;
    if ((rc = finish(out, write_points(out, "Particles by Mass", group[g]), path)) != GG_OK) return rc;
  }
  return GG_OK;
}

// saveFunnelBoundaryParticlesToVTK (main.cu:370-432, centred = 0) and
// saveBoundaryParticlesToVTK (main.cu:434-527, centred = 1: centred on the
// valid render points): the animated wall particles.  The file is created
// even when no wall particle is animated (then empty).
gg_status gg_write_vtk_animated_boundary(gg_system* S, const char* path, int32_t centred) {
  if (!S || !path) {
    gg::set_error("gg_write_vtk_animated_boundary: null argument");
    return GG_ERR_INVALID_ARGUMENT;
  }
  std::ofstream out;
  gg_status rc = open_out(path, out);
  if (rc != GG_OK) return rc;
  std::vector<F3> walls;
  if ((rc = animated_walls(S, walls)) != GG_OK) return rc;
  if (walls.empty()) return finish(out, true, path);
  if (centred) {
    std::vector<F3> up;
    if ((rc = read_pos(S, GG_SET_UPSAMPLED, up)) != GG_OK) return rc;
    const Centring t = centring_of(valid_only(up), true);
    for (F3& p : walls) p = t.apply(p);
  }
  return finish(out, write_points(out, "Animated Boundary Particles", walls), path);
}

// saveAdditionalBoundaryParticlesToVTK (main.cu:529-586): host points
// (float[3] each), centred on the valid render points.
gg_status gg_write_vtk_points_centered(gg_system* S, const float* points3, int64_t n, const char* path) {
  if (!S || !path || n < 0 || (n > 0 && !points3)) {
    gg::set_error("gg_write_vtk_points_centered: null argument or negative count");
    return GG_ERR_INVALID_ARGUMENT;
  }
  std::ofstream out;
  gg_status rc = open_out(path, out);
  if (rc != GG_OK) return rc;
  std::vector<F3> up;
  if ((rc = read_pos(S, GG_SET_UPSAMPLED, up)) != GG_OK) return rc;
  const Centring t = centring_of(valid_only(up), true);
  std::vector<F3> pts((size_t)n);
  for (int64_t i = 0; i < n; ++i) pts[(size_t)i] = t.apply({points3[3 * i], points3[3 * i + 1], points3[3 * i + 2]});
  return finish(out, write_points(out, "Additional Boundary Particles", pts), path);
}

// saveUpsampledPositionsToCSV (main.cu:673-694): "x,y,z" per point, every
// point as stored.
gg_status gg_write_csv(gg_system* S, gg_set set, const char* path) {
  if (!S || !path) {
    gg::set_error("gg_write_csv: null argument");
    return GG_ERR_INVALID_ARGUMENT;
  }
  std::vector<F3> pos;
  gg_status rc = read_pos(S, set, pos);
  if (rc != GG_OK) return rc;
  std::ofstream out;
  if ((rc = open_out(path, out)) != GG_OK) return rc;
  for (const F3& p : pos) out << p.x << "," << p.y << "," << p.z << "\n";
  return finish(out, true, path);
}

// saveFrameTimes (main.cu:665-671): one device-millisecond figure per line.
gg_status gg_write_frame_times(gg_system* S, const char* path) {
  if (!S || !path) {
    gg::set_error("gg_write_frame_times: null argument");
    return GG_ERR_INVALID_ARGUMENT;
  }
  int64_t n = 0;
  gg_status rc = gg_frame_times(S, nullptr, 0, &n);
  if (rc != GG_OK) return rc;
  std::vector<float> t((size_t)n);
  if (n && (rc = gg_frame_times(S, t.data(), n, &n)) != GG_OK) return rc;
  std::ofstream out;
  if ((rc = open_out(path, out)) != GG_OK) return rc;
  for (float v : t) out << v << "\n";
  return finish(out, true, path);
}

}  // extern "C"
