// Named host callbacks registered through the C-ABI
// (src/core/util/callback_manager.cpp; src/core/extern.cpp add_*_callback).
#pragma once
#include <map>
#include <mutex>
#include <string>

#include "props.h"

namespace sg {

using IoCallback = void (*)(int id, int size, void* data);
using WeightCallback = void (*)(int id, int size, void* weights);
using IndicesCallback = void (*)(int id, int size, void* weights, void* from_indices,
                                 void* to_indices, void* used);
using DistanceCallback = void (*)(int id, int size, void* weights, void* distances);
using DelayCallback = void (*)(int id, int size, void* weights, void* delays);

class Callbacks {
  public:
    static Callbacks& get() {
        static Callbacks c;
        return c;
    }
    std::map<std::string, IoCallback> io;
    std::map<std::string, WeightCallback> weight;
    std::map<std::string, IndicesCallback> indices;
    std::map<std::string, DistanceCallback> distance;
    std::map<std::string, DelayCallback> delay;

    template <class T>
    static T find(const std::map<std::string, T>& m, const std::string& name, const char* kind) {
        auto it = m.find(name);
        if (it == m.end()) throw SgError(std::string("Unrecognized ") + kind + " callback: " + name);
        return it->second;
    }
};

}  // namespace sg
