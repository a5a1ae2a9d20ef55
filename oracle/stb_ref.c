/* The reference's vendored BC1 encoder (o-bc1/stb_dxt.h, v1.08b), compiled from
 * where it lies in the vkdt tree into oracle/_ref/libstb_dxt.so by
 * oracle.build_stb_ref(). TEST INFRASTRUCTURE ONLY: it pins the BC1
 * restatement in oracle.cpp (and the fixtures made from it). */
#define STB_DXT_IMPLEMENTATION
#include "stb_dxt.h"

/* o-bc1/main.c:30-47: every whole 4x4 block of an rgba u8 image, no alpha, normal mode */
void stb_ref_bc1(const unsigned char *rgba, int wd, int ht, unsigned char *out)
{
  const int bx = wd / 4, by = ht / 4;
  for(int j = 0; j < 4 * by; j += 4)
    for(int i = 0; i < 4 * bx; i += 4)
    {
      unsigned char block[64];
      for(int jj = 0; jj < 4; jj++)
        for(int ii = 0; ii < 4; ii++)
          for(int c = 0; c < 4; c++)
            block[4 * (4 * jj + ii) + c] = rgba[4 * (wd * (j + jj) + (i + ii)) + c];
      stb_compress_dxt_block(out + 8 * (bx * (j / 4) + (i / 4)), block, 0, 0);
    }
}
