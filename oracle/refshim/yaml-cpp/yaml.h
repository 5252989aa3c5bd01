// Stand-in for the yaml-cpp names that core/Common.h mentions (TEST INFRASTRUCTURE for oracle/_ref).
#pragma once
namespace YAML {
struct EmitterStyle {
    enum value { Default, Block, Flow };
};
class Node {
  public:
    template <class T> void push_back(const T &) {}
    void SetStyle(EmitterStyle::value) {}
};
template <class T> struct convert;
} // namespace YAML
