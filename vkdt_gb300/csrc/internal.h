// Host-side declarations shared by the translation units of libvkdt_cuda
// (not part of the C-ABI).
#pragma once

// set the calling thread's vkdt_cuda_last_error() text; returns code
int vkdt_set_error(int code, const char *msg);
