// Stand-in for <GL/glew.h>: the reference's headers only need the GL integer
// typedefs to declare buffer handles.  No GL function is declared or called.
#pragma once
typedef unsigned int GLuint;
typedef int GLint;
typedef unsigned int GLenum;
