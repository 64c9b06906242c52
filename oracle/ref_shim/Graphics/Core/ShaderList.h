// ShaderList.h stand-in for the reference pin (oracle/_ref, test
// infrastructure only).  NaiveFracturer.cpp's GPU methods name the OpenGL
// compute-shader wrapper; the pin calls only the CPU path (buildCPU), so
// these members exist to let the file compile and are never called.
#pragma once
#include "stdafx.h"

typedef unsigned int GLenum;
#define GL_DYNAMIC_DRAW 0x88E8
#define GL_STATIC_DRAW 0x88E4
#define GL_COMPUTE_SHADER 0x91B9

namespace RendEnum {
enum ComputeShaderTypes { NAIVE_FRACTURER, REMOVE_ISOLATED_REGIONS };
}

class ComputeShader {
 public:
  static unsigned getNumGroups(unsigned) { return 1; }
  static unsigned getMaxGroupSize() { return 1; }
  template <typename T> static GLuint setWriteBuffer(const T&, size_t, GLenum) { return 0; }
  template <typename T> static GLuint setReadBuffer(const T*, size_t, GLenum) { return 0; }
  template <typename T> static GLuint setReadBuffer(const std::vector<T>&, GLenum) { return 0; }
  template <typename T> static void updateReadBuffer(GLuint, const T*, size_t, GLenum) {}
  template <typename T> static void updateReadBufferSubset(GLuint, const T*, size_t, size_t) {}
  template <typename T> static T* readData(GLuint, const T&) { return nullptr; }
  static void deleteBuffer(GLuint) {}
  static void deleteBuffers(const std::vector<GLuint>&) {}
  void bindBuffers(const std::vector<GLuint>&) {}
  void use() {}
  template <typename T> void setUniform(const std::string&, const T&) {}
  void setSubroutineUniform(GLenum, const std::string&, const std::string&) {}
  void applyActiveSubroutines() {}
  void execute(unsigned, unsigned, unsigned, unsigned, unsigned, unsigned) {}
};

class ShaderList {
 public:
  static ShaderList* getInstance() {
    static ShaderList s;
    return &s;
  }
  ComputeShader* getComputeShader(RendEnum::ComputeShaderTypes) {
    static ComputeShader c;
    return &c;
  }
};
