// scene.h — the reference's scene-JSON format and scene construction.
#pragma once

#include <stdint.h>

#include <map>
#include <memory>
#include <string>
#include <vector>

#include "../../include/gg.h"

namespace gg {

// Minimal JSON value: objects, arrays, numbers, strings, booleans, null.
struct Json {
  enum Kind { Null, Bool, Number, String, Array, Object } kind = Null;
  double num = 0.0;
  bool b = false;
  std::string str;
  std::vector<Json> arr;
  std::map<std::string, Json> obj;
  const Json* get(const std::string& k) const {
    auto it = obj.find(k);
    return it == obj.end() ? nullptr : &it->second;
  }
};

// Parses text; returns false with a message on malformed input.
bool json_parse(const std::string& text, Json& out, std::string& err);

// AnimationState's initialisers (animation.cu).
void default_animation(gg_animation* a);

// The particle sets and constructor arguments init_granular_system
// (main.cu:746-1173) builds from a scene file, and the animation state it
// leaves.
struct SceneData {
  std::vector<float> particles;   // float[3] each
  std::vector<float> boundary;
  std::vector<int32_t> animated;
  std::vector<float> upsampled;
  gg_desc desc{};
  std::string save_file;
  gg_animation animation{};
  SceneData() { default_animation(&animation); }
};

gg_status scene_build(const char* json_path, const char* base_dir, SceneData& out);

}  // namespace gg
