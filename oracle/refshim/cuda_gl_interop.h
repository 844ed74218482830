/* Host shim: empty stand-in (the reference kernels compiled as host code need nothing from this header). */
#pragma once
