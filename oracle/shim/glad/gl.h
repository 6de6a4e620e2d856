// Shim for the reference build only (oracle/_ref): the two GL names the reference's CPU solver files
// mention in their (never called) OpenGL solver classes.
#pragma once
typedef unsigned int GLuint;
#define GL_SHADER_STORAGE_BARRIER_BIT 0x00002000
inline void glMemoryBarrier(unsigned int) {}
