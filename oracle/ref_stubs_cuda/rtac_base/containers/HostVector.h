// Stand-in for rtac_base HostVector<T>.
#pragma once
#include <vector>
namespace rtac { template <typename T> using HostVector = std::vector<T>; }
