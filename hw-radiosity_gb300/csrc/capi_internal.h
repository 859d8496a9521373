// Definitions of the opaque C-ABI handles (internal).
#pragma once
#include <string>

#include "rad_host.h"

struct rad_scene {
    int precision = 32;
    radgb::Scene<float> s32;
    radgb::Scene<double> s64;
    std::string log_out, log_err;   // last call's info lines, split by stream
};

struct rad_octree {
    int precision = 32;
    radgb::Octree<float> o32;
    radgb::Octree<double> o64;
};

namespace radgb {
void set_error(const std::string& msg);
int fail(int code, const std::string& msg);
// move the scene's info lines into the handle (stdout / stderr streams)
void take_scene_log(rad_scene* h);
}  // namespace radgb
