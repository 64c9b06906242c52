// Model3D.h stand-in for the reference pin (oracle/_ref, test infrastructure
// only): Triangle3D.h names Model3D's GPU vertex and face records; the real
// header needs OpenGL.  The fields are the ones Triangle3D.cpp touches.
#pragma once
#include "stdafx.h"

class Model3D {
 public:
  struct VertexGPUData {
    vec3 _position, _normal;
    vec2 _textCoord;
    vec3 _tangent;
  };
  struct FaceGPUData {
    uvec3 _vertices;
    unsigned _modelCompID;
    vec3 _minPoint, _maxPoint, _normal;
  };
};
