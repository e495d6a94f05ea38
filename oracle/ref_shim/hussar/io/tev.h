// ORACLE — TEST INFRASTRUCTURE ONLY.
// Stands in for libhussar/include/hussar/io/tev.h (debug-image streaming to the tev
// viewer over a socket, off the hot path): the names integrator.h uses, doing nothing.
#pragma once
#include <string>

#include <hussar/io/exr.h>

namespace hussar {

class TevStream : public Channelizer {
public:
    TevStream(const std::string &) {}
    template <typename T> void add(Image<T> &, ChannelName = ChannelName()) {}
    void stream() {}
};

}  // namespace hussar
