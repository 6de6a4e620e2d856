// Shim for the reference build only (oracle/_ref): the reference's Shader (include/assets/Shader.h)
// reduced to the calls its OpenGL solver classes make, with no-op bodies; those classes are never used.
#pragma once
#include <initializer_list>
#include <string>
#include <utility>
#include "glad/gl.h"
class Shader {
public:
    enum Type { VERTEX, FRAGMENT, COMPUTE, COUNT };
    Shader() = default;
    Shader(std::initializer_list<std::pair<std::string, Type>>, bool = true) {}
    void bind() const {}
    void unbind() const {}
    void dispatch(unsigned int, unsigned int = 1, unsigned int = 1) const {}
    void setFloat(const std::string&, float) const {}
    void setInt(const std::string&, int) const {}
    void setUInt(const std::string&, unsigned int) const {}
    void setBool(const std::string&, bool) const {}
};
