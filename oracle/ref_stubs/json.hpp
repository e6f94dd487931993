/* Declaration-only stand-in for nlohmann::json, enough for the reference's
 * config header to parse when its simulation source is compiled for the
 * device. Nothing here is defined or called. Test infrastructure only. */
#pragma once
#include <string>
namespace nlohmann {
struct json {
  bool contains(const std::string&) const;
  json at(const std::string&) const;
  template <class T> operator T() const;
};
}  // namespace nlohmann
