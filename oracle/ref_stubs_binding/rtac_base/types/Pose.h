// Stand-in for rtac_base types/Pose.h: only the type is used by the sensor
// headers the binding compiles against.
#pragma once
namespace rtac { template <typename T> struct Pose { T position[3] = {0, 0, 0}; T orientation[4] = {1, 0, 0, 0}; }; }
