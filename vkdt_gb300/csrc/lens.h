// the lens node (lens/main.comp): its uniform block and launcher (k_nodes.cu)
#pragma once
#include <cuda_runtime.h>

struct half4;
// lens/main.comp:9-15, in the order of lens/params: centre, scale, the two sphere radii, ca red/blue
struct lens_par_t { float c[2], f[2], r[2], ca[2]; };
// lens/main.comp on a w x h rgba f16 image into ow x oh
cudaError_t launch_lens(const half4 *in, int w, int h, half4 *out, int ow, int oh, const lens_par_t &q, cudaStream_t s);
