// config_parser.hpp — the reference's configuration loader
// (class ConfigParser, inc/config_parser.hpp:118-151; defaults and keys,
// src/config_parser.cpp:11-184) on a small JSON reader of this project, so
// that a host program that reads OpenSayal.conf.json (src/main.cu:42-49)
// builds unchanged:
//
//   Config config = ConfigParser().parse();        // ./OpenSayal.conf.json
//   Config config = ConfigParser("my.json").parse();
//
// Lookup follows ConfigParser::get_or exactly: a dotted key is first looked
// up whole at the current level; otherwise it is split at its FIRST dot and
// the rest is looked up inside the member named by the part before it.
// Conversions follow the JSON library the reference uses: numbers convert to
// int by truncation and to float by rounding, booleans convert to numbers,
// and a boolean key needs a JSON boolean. When a value of the wrong type is
// found inside a nested object, the reference's catch-all around the
// recursion turns the error into the default, and so does this parser; a
// wrong type for a key given whole at the top level is an error.
//
// Differences a caller can observe: errors (an unreadable file, malformed
// JSON, a wrong top-level type) throw opensayal::Error instead of ending the
// program through an uncaught exception; thread.openMP.thread_count defaults
// to 0 (the reference's default, omp_get_thread_num() / 2 outside a parallel
// region, is 0 as well).
//
// Header-only C++17 with no dependency beyond the standard library and the
// C ABI header; the library's os_config_parse (C ABI) is built on the same
// reader. Including it defines the reference's Config structs
// (inc/config_parser.hpp:9-115).
#pragma once

#include <algorithm>
#include <cerrno>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <memory>
#include <sstream>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "../opensayal_gb300.h"

// --- inc/config_parser.hpp:9-115 -------------------------------------------
struct ColorConfig { int r; int g; int b; int a; };
struct OpenMPConfig { int thread_count; };
struct CudaConfig { int block_size_x; int block_size_y; };
struct ThreadConfig { OpenMPConfig openMP; CudaConfig cuda; };
struct ProjectionConfig { int n; float o; };
struct PhysicsConfig { float g; };
struct WindTunnelConfig {
  int pipe_height; int pipe_length; int smoke_length; int smoke_height; int smoke_count;
  float speed; float smoke;
};
struct ObstacleConfig { bool enable; int center_x; int center_y; float radius; };
struct TimeConfig { float d_t; bool enable_real_time; float real_time_multiplier; };
struct SmokeConfig { bool enable_decay; float decay_rate; };
struct PathLineConfig { bool enable; int length; ColorConfig color; int distance; };
struct FluidConfig { float density; float drag_coeff; float viscosity; };
struct SimConfig {
  int height; int width; int cell_pixel_size; float cell_size;
  bool enable_drain; bool enable_pressure; bool enable_smoke; bool enable_interactive;
  ProjectionConfig projection; WindTunnelConfig wind_tunnel; PhysicsConfig physics;
  TimeConfig time; SmokeConfig smoke; ObstacleConfig obstacle;
};
struct ArrowConfig {
  ColorConfig color; bool enable; int distance; float length_multiplier;
  float disable_threshold; int head_length;
};
struct VisualConfig { ArrowConfig arrows; PathLineConfig path_line; };
struct Config { ThreadConfig thread; SimConfig sim; FluidConfig fluid; VisualConfig visual; };

namespace opensayal {

struct Error : std::runtime_error {
  int code;
  Error(int c, const std::string& what) : std::runtime_error(what), code(c) {}
};

inline void check(int rc) {
  if (rc != OS_OK) throw Error(rc, os_last_error());
}

namespace json {

// A parsed JSON value. Numbers keep whether they were written as integers
// (no fraction or exponent), as the reference's JSON library does, so that an
// integer too large for a double keeps its exact value.
struct Value {
  enum class Kind { Null, Bool, Int, UInt, Float, String, Array, Object };
  Kind kind = Kind::Null;
  bool b = false;
  int64_t i = 0;
  uint64_t u = 0;
  double f = 0.0;
  std::string s;
  std::vector<Value> items;
  std::vector<std::pair<std::string, Value>> members;

  bool is_object() const { return kind == Kind::Object; }
  bool is_number() const {
    return kind == Kind::Int || kind == Kind::UInt || kind == Kind::Float;
  }

  // The member named `key` (the last one when a key repeats), or nullptr.
  const Value* find(const std::string& key) const {
    if (kind != Kind::Object) return nullptr;
    for (auto it = members.rbegin(); it != members.rend(); ++it)
      if (it->first == key) return &it->second;
    return nullptr;
  }
};

struct ParseError : std::runtime_error {
  explicit ParseError(const std::string& m) : std::runtime_error(m) {}
};

struct TypeError : std::runtime_error {
  explicit TypeError(const std::string& m) : std::runtime_error(m) {}
};

// Strict RFC 8259 reader: one value with optional surrounding whitespace.
class Reader {
 public:
  explicit Reader(const std::string& text) : p_(text.data()), end_(text.data() + text.size()),
                                             begin_(text.data()) {}

  Value parse() {
    Value v = value(0);
    ws();
    if (p_ != end_) fail("trailing characters after the JSON value");
    return v;
  }

 private:
  const char* p_;
  const char* end_;
  const char* begin_;
  static constexpr int kMaxDepth = 256;

  [[noreturn]] void fail(const std::string& what) const {
    throw ParseError("JSON: " + what + " at offset " + std::to_string(p_ - begin_));
  }

  void ws() {
    while (p_ != end_ && (*p_ == ' ' || *p_ == '\t' || *p_ == '\n' || *p_ == '\r')) ++p_;
  }

  bool literal(const char* word) {
    size_t n = std::strlen(word);
    if ((size_t)(end_ - p_) >= n && std::memcmp(p_, word, n) == 0) {
      p_ += n;
      return true;
    }
    return false;
  }

  Value value(int depth) {
    if (depth > kMaxDepth) fail("nesting too deep");
    ws();
    if (p_ == end_) fail("unexpected end of input");
    Value v;
    switch (*p_) {
      case '{': return object(depth);
      case '[': return array(depth);
      case '"': v.kind = Value::Kind::String; v.s = string(); return v;
      case 't': if (literal("true")) { v.kind = Value::Kind::Bool; v.b = true; return v; } break;
      case 'f': if (literal("false")) { v.kind = Value::Kind::Bool; v.b = false; return v; } break;
      case 'n': if (literal("null")) return v; break;
      default:
        if (*p_ == '-' || (*p_ >= '0' && *p_ <= '9')) return number();
    }
    fail("unexpected character");
  }

  Value object(int depth) {
    Value v;
    v.kind = Value::Kind::Object;
    ++p_;  // '{'
    ws();
    if (p_ != end_ && *p_ == '}') { ++p_; return v; }
    for (;;) {
      ws();
      if (p_ == end_ || *p_ != '"') fail("expected a member name");
      std::string key = string();
      ws();
      if (p_ == end_ || *p_ != ':') fail("expected ':'");
      ++p_;
      v.members.emplace_back(std::move(key), value(depth + 1));
      ws();
      if (p_ == end_) fail("unterminated object");
      if (*p_ == ',') { ++p_; continue; }
      if (*p_ == '}') { ++p_; return v; }
      fail("expected ',' or '}'");
    }
  }

  Value array(int depth) {
    Value v;
    v.kind = Value::Kind::Array;
    ++p_;  // '['
    ws();
    if (p_ != end_ && *p_ == ']') { ++p_; return v; }
    for (;;) {
      v.items.push_back(value(depth + 1));
      ws();
      if (p_ == end_) fail("unterminated array");
      if (*p_ == ',') { ++p_; continue; }
      if (*p_ == ']') { ++p_; return v; }
      fail("expected ',' or ']'");
    }
  }

  unsigned hex4() {
    if (end_ - p_ < 4) fail("short \\u escape");
    unsigned cp = 0;
    for (int k = 0; k < 4; k++) {
      char c = *p_++;
      cp <<= 4;
      if (c >= '0' && c <= '9') cp |= (unsigned)(c - '0');
      else if (c >= 'a' && c <= 'f') cp |= (unsigned)(c - 'a' + 10);
      else if (c >= 'A' && c <= 'F') cp |= (unsigned)(c - 'A' + 10);
      else fail("bad hex digit in \\u escape");
    }
    return cp;
  }

  static void utf8(std::string& out, unsigned cp) {
    if (cp < 0x80) {
      out += (char)cp;
    } else if (cp < 0x800) {
      out += (char)(0xC0 | (cp >> 6));
      out += (char)(0x80 | (cp & 0x3F));
    } else if (cp < 0x10000) {
      out += (char)(0xE0 | (cp >> 12));
      out += (char)(0x80 | ((cp >> 6) & 0x3F));
      out += (char)(0x80 | (cp & 0x3F));
    } else {
      out += (char)(0xF0 | (cp >> 18));
      out += (char)(0x80 | ((cp >> 12) & 0x3F));
      out += (char)(0x80 | ((cp >> 6) & 0x3F));
      out += (char)(0x80 | (cp & 0x3F));
    }
  }

  std::string string() {
    ++p_;  // opening quote
    std::string out;
    for (;;) {
      if (p_ == end_) fail("unterminated string");
      unsigned char c = (unsigned char)*p_++;
      if (c == '"') return out;
      if (c < 0x20) fail("control character in string");
      if (c != '\\') { out += (char)c; continue; }
      if (p_ == end_) fail("unterminated escape");
      char e = *p_++;
      switch (e) {
        case '"': out += '"'; break;
        case '\\': out += '\\'; break;
        case '/': out += '/'; break;
        case 'b': out += '\b'; break;
        case 'f': out += '\f'; break;
        case 'n': out += '\n'; break;
        case 'r': out += '\r'; break;
        case 't': out += '\t'; break;
        case 'u': {
          unsigned cp = hex4();
          if (cp >= 0xD800 && cp <= 0xDBFF) {
            if (end_ - p_ < 2 || p_[0] != '\\' || p_[1] != 'u') fail("unpaired surrogate");
            p_ += 2;
            unsigned lo = hex4();
            if (lo < 0xDC00 || lo > 0xDFFF) fail("bad low surrogate");
            cp = 0x10000 + ((cp - 0xD800) << 10) + (lo - 0xDC00);
          } else if (cp >= 0xDC00 && cp <= 0xDFFF) {
            fail("unpaired surrogate");
          }
          utf8(out, cp);
          break;
        }
        default: fail("bad escape");
      }
    }
  }

  Value number() {
    const char* start = p_;
    bool integral = true;
    if (*p_ == '-') ++p_;
    if (p_ == end_) fail("bad number");
    if (*p_ == '0') {
      ++p_;
    } else if (*p_ >= '1' && *p_ <= '9') {
      while (p_ != end_ && *p_ >= '0' && *p_ <= '9') ++p_;
    } else {
      fail("bad number");
    }
    if (p_ != end_ && *p_ == '.') {
      integral = false;
      ++p_;
      if (p_ == end_ || !(*p_ >= '0' && *p_ <= '9')) fail("bad fraction");
      while (p_ != end_ && *p_ >= '0' && *p_ <= '9') ++p_;
    }
    if (p_ != end_ && (*p_ == 'e' || *p_ == 'E')) {
      integral = false;
      ++p_;
      if (p_ != end_ && (*p_ == '+' || *p_ == '-')) ++p_;
      if (p_ == end_ || !(*p_ >= '0' && *p_ <= '9')) fail("bad exponent");
      while (p_ != end_ && *p_ >= '0' && *p_ <= '9') ++p_;
    }
    std::string text(start, p_);
    Value v;
    if (integral) {
      errno = 0;
      if (*start == '-') {
        long long x = std::strtoll(text.c_str(), nullptr, 10);
        if (errno == 0) {
          v.kind = Value::Kind::Int;
          v.i = x;
          return v;
        }
      } else {
        unsigned long long x = std::strtoull(text.c_str(), nullptr, 10);
        if (errno == 0) {
          v.kind = Value::Kind::UInt;
          v.u = x;
          return v;
        }
      }
      // beyond 64 bits: kept as a floating-point number
    }
    v.kind = Value::Kind::Float;
    v.f = std::strtod(text.c_str(), nullptr);  // correctly rounded (C locale digits)
    return v;
  }
};

inline Value parse(const std::string& text) { return Reader(text).parse(); }

// The conversions get_or applies to a found value.
inline int to_int(const Value& v) {
  switch (v.kind) {
    case Value::Kind::Int: return static_cast<int>(v.i);
    case Value::Kind::UInt: return static_cast<int>(v.u);
    case Value::Kind::Float: return static_cast<int>(v.f);
    case Value::Kind::Bool: return v.b ? 1 : 0;
    default: throw TypeError("type must be number");
  }
}

inline float to_float(const Value& v) {
  switch (v.kind) {
    case Value::Kind::Int: return static_cast<float>(v.i);
    case Value::Kind::UInt: return static_cast<float>(v.u);
    case Value::Kind::Float: return static_cast<float>(v.f);
    case Value::Kind::Bool: return v.b ? 1.0f : 0.0f;
    default: throw TypeError("type must be number");
  }
}

inline bool to_bool(const Value& v) {
  if (v.kind != Value::Kind::Bool) throw TypeError("type must be boolean");
  return v.b;
}

template <typename T>
T convert(const Value& v);
template <>
inline int convert<int>(const Value& v) { return to_int(v); }
template <>
inline float convert<float>(const Value& v) { return to_float(v); }
template <>
inline bool convert<bool>(const Value& v) { return to_bool(v); }

// ConfigParser::get_or (inc/config_parser.hpp:131-150). `top` says whether
// this is the outermost call: a conversion error there propagates (the
// reference lets it escape), one below it yields the default (the reference's
// catch-all around the recursion).
template <typename T>
T get_or(const Value& obj, const std::string& key, T default_value, bool top = true) {
  if (const Value* found = obj.find(key)) {
    if (top) return convert<T>(*found);
    try {
      return convert<T>(*found);
    } catch (const TypeError&) {
      return default_value;
    }
  }
  if (key.empty()) return default_value;
  const size_t dot = key.find('.');
  if (dot == std::string::npos) return default_value;
  const Value* child = obj.find(key.substr(0, dot));
  if (!child) return default_value;
  return get_or<T>(*child, key.substr(dot + 1), default_value, false);
}

}  // namespace json
}  // namespace opensayal

namespace opensayal {
// Fill the reference's Config from a parsed document
// (src/config_parser.cpp:21-179, in the order the reference reads the keys).
inline Config config_from_json(const json::Value& j) {
  using json::get_or;
  Config c{};
  const int sim_height = get_or(j, "sim.height", 1080);
  const int sim_width = get_or(j, "sim.width", 1920);
  c.thread.openMP.thread_count = get_or(j, "thread.openMP.thread_count", 0);
  c.thread.cuda.block_size_x = get_or(j, "thread.cuda.block_size_x", 64);
  c.thread.cuda.block_size_y = get_or(j, "thread.cuda.block_size_y", 1);
  c.sim.height = sim_height;
  c.sim.width = sim_width;
  c.sim.cell_pixel_size = get_or(j, "sim.cell_pixel_size", 1);
  c.sim.cell_size = get_or(j, "sim.cell_size", 1.0f);
  c.sim.enable_drain = get_or(j, "sim.enable_drain", true);
  c.sim.enable_pressure = get_or(j, "sim.enable_pressure", false);
  c.sim.enable_smoke = get_or(j, "sim.enable_smoke", true);
  c.sim.enable_interactive = get_or(j, "sim.enable_interactive", false);
  c.sim.projection.n = get_or(j, "sim.projection.n", 50);
  c.sim.projection.o = get_or(j, "sim.projection.o", 1.9f);
  c.sim.wind_tunnel.pipe_height = get_or(j, "sim.wind_tunnel.pipe_height", sim_height / 4);
  c.sim.wind_tunnel.pipe_length = 0;
  c.sim.wind_tunnel.smoke_length = get_or(j, "sim.wind_tunnel.smoke_length", 1);
  c.sim.wind_tunnel.smoke_height = get_or(j, "sim.wind_tunnel.smoke_height", sim_height / 4);
  c.sim.wind_tunnel.smoke_count = get_or(j, "sim.wind_tunnel.smoke_count", 1);
  c.sim.wind_tunnel.speed = get_or(j, "sim.wind_tunnel.speed", 0.0f);
  c.sim.wind_tunnel.smoke = get_or(j, "sim.wind_tunnel.smoke", 1.0f);
  c.sim.physics.g = get_or(j, "sim.physics.g", 0.0f);
  c.sim.time.d_t = get_or(j, "sim.time.d_t", 0.05f);
  c.sim.time.enable_real_time = get_or(j, "sim.time.enable_real_time", false);
  c.sim.time.real_time_multiplier = get_or(j, "sim.time.real_time_multiplier", 1.0f);
  c.sim.smoke.enable_decay = get_or(j, "sim.smoke.enable_decay", false);
  c.sim.smoke.decay_rate = get_or(j, "sim.smoke.decay_rate", 0.05f);
  c.sim.obstacle.enable = get_or(j, "sim.obstacle.enable", true);
  c.sim.obstacle.center_x = get_or(j, "sim.obstacle.center_x", sim_width / 2);
  c.sim.obstacle.center_y = get_or(j, "sim.obstacle.center_y", sim_height / 2);
  c.sim.obstacle.radius = get_or(j, "sim.obstacle.radius",
                                 std::min(sim_height, sim_width) / 30.0f);
  c.fluid.density = get_or(j, "fluid.density", 1.0f);
  c.fluid.drag_coeff = get_or(j, "fluid.drag_coeff", 0.0f);
  c.fluid.viscosity = get_or(j, "fluid.viscosity", 0.001f);
  c.visual.arrows.color.r = get_or(j, "visual.arrows.color.r", 0);
  c.visual.arrows.color.g = get_or(j, "visual.arrows.color.g", 0);
  c.visual.arrows.color.b = get_or(j, "visual.arrows.color.b", 0);
  c.visual.arrows.color.a = get_or(j, "visual.arrows.color.a", 255);
  c.visual.arrows.enable = get_or(j, "visual.arrows.enable", false);
  c.visual.arrows.distance = get_or(j, "visual.arrows.distance", 20);
  c.visual.arrows.length_multiplier = get_or(j, "visual.arrows.length_multiplier", 0.1f);
  c.visual.arrows.disable_threshold = get_or(j, "visual.arrows.disable_threshold", 0.0f);
  c.visual.arrows.head_length = get_or(j, "visual.arrows.head_length", 5);
  c.visual.path_line.enable = get_or(j, "visual.path_line.enable", false);
  c.visual.path_line.length = get_or(j, "visual.path_line.length", 20);
  c.visual.path_line.color.r = get_or(j, "visual.path_line.color.r", 0);
  c.visual.path_line.color.g = get_or(j, "visual.path_line.color.g", 0);
  c.visual.path_line.color.b = get_or(j, "visual.path_line.color.b", 0);
  c.visual.path_line.color.a = get_or(j, "visual.path_line.color.a", 255);
  c.visual.path_line.distance = get_or(j, "visual.path_line.distance", 20);
  return c;
}

// Config -> os_config (every key the simulation reads; the library's own
// fields keep os_config_defaults' values: F32 storage, autotuned depths).
inline int to_os_config(const Config& c, os_config* o) {
  const int rc = os_config_defaults(c.sim.width, c.sim.height, o);
  if (rc != OS_OK) return rc;
  o->block_size_x = c.thread.cuda.block_size_x;
  o->block_size_y = c.thread.cuda.block_size_y;
  o->cell_pixel_size = c.sim.cell_pixel_size;
  o->cell_size = c.sim.cell_size;
  o->enable_drain = c.sim.enable_drain;
  o->enable_pressure = c.sim.enable_pressure;
  o->enable_smoke = c.sim.enable_smoke;
  o->enable_interactive = c.sim.enable_interactive;
  o->projection_n = c.sim.projection.n;
  o->projection_o = c.sim.projection.o;
  o->pipe_height = c.sim.wind_tunnel.pipe_height;
  o->pipe_length = c.sim.wind_tunnel.pipe_length;
  o->smoke_length = c.sim.wind_tunnel.smoke_length;
  o->smoke_height = c.sim.wind_tunnel.smoke_height;
  o->smoke_count = c.sim.wind_tunnel.smoke_count;
  o->tunnel_speed = c.sim.wind_tunnel.speed;
  o->tunnel_smoke = c.sim.wind_tunnel.smoke;
  o->g = c.sim.physics.g;
  o->d_t = c.sim.time.d_t;
  o->enable_real_time = c.sim.time.enable_real_time;
  o->real_time_multiplier = c.sim.time.real_time_multiplier;
  o->smoke_enable_decay = c.sim.smoke.enable_decay;
  o->smoke_decay_rate = c.sim.smoke.decay_rate;
  o->obstacle_enable = c.sim.obstacle.enable;
  o->obstacle_center_x = c.sim.obstacle.center_x;
  o->obstacle_center_y = c.sim.obstacle.center_y;
  o->obstacle_radius = c.sim.obstacle.radius;
  o->density = c.fluid.density;
  o->drag_coeff = c.fluid.drag_coeff;
  o->viscosity = c.fluid.viscosity;
  return OS_OK;
}

// Config -> os_visual_config (the keys the headless visuals read).
inline void to_os_visual_config(const Config& c, os_visual_config* v) {
  std::memset(v, 0, sizeof *v);
  v->cell_pixel_size = c.sim.cell_pixel_size;
  v->arrow_distance = c.visual.arrows.distance;
  v->arrow_length_multiplier = c.visual.arrows.length_multiplier;
  v->arrow_disable_threshold = c.visual.arrows.disable_threshold;
  v->arrow_head_length = c.visual.arrows.head_length;
  v->trace_distance = c.visual.path_line.distance;
  v->trace_length = c.visual.path_line.length;
}
}  // namespace opensayal

// ConfigParser (inc/config_parser.hpp:118-129): the file name defaults to
// OpenSayal.conf.json in the working directory (src/config_parser.cpp:13).
class ConfigParser {
 private:
  const std::string config_file_name;

 public:
  explicit ConfigParser(std::string config_file_name)
      : config_file_name(std::move(config_file_name)) {}
  ConfigParser() : config_file_name("OpenSayal.conf.json") {}

  Config parse() const {
    std::ifstream in(config_file_name, std::ios::binary);
    if (!in) throw opensayal::Error(OS_ERR_INVALID, "cannot open " + config_file_name);
    std::stringstream ss;
    ss << in.rdbuf();
    try {
      return opensayal::config_from_json(opensayal::json::parse(ss.str()));
    } catch (const opensayal::json::ParseError& e) {
      throw opensayal::Error(OS_ERR_INVALID, config_file_name + ": " + e.what());
    } catch (const opensayal::json::TypeError& e) {
      throw opensayal::Error(OS_ERR_INVALID, config_file_name + ": " + e.what());
    }
  }
};
