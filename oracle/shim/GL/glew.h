// Test infrastructure only.  Type names the reference headers mention
// (SPHSystem.h, Geometry.h) so that the physics translation units compile
// headless.  No graphics function is declared or provided: the oracle build
// compiles only src/sph.cpp, src/neighborTable.cpp and src/timer.cpp, none of
// which calls into a graphics API.
#pragma once
typedef unsigned int GLuint;
typedef unsigned int GLenum;
typedef int GLint;
typedef float GLfloat;
