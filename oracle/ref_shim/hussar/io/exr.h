// ORACLE — TEST INFRASTRUCTURE ONLY.
// Stands in for libhussar/include/hussar/io/exr.h (debug-image EXR output through
// tinyexr, absent here and off the hot path): the names integrator.h uses, doing nothing.
#pragma once
#include <string>

#include <hussar/core/image.h>

namespace hussar {

class Channelizer {
public:
    struct ChannelName {
        std::string name;
        ChannelName() {}
        ChannelName(const std::string &n) : name(n) {}
    };
};

class ExrSaveFile : public Channelizer {
public:
    ExrSaveFile(const std::string &) {}
    template <typename T> void add(Image<T> &, ChannelName = ChannelName()) {}
    void save() {}
};

}  // namespace hussar
