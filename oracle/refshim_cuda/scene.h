/* CUDA-build shim: empty stand-in.  The reference kernels compiled by nvcc
 * (oracle/ref_cuda.cu) need nothing from this header; its real counterpart
 * pulls in OpenGL, Windows console or scene-loading code. */
#pragma once
