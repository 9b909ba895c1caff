/* Runs the reference's generate_rotation_list (rotations.c:77-458, compiled
 * unchanged from the reference tree by oracle/build_ref.sh) and writes
 * int32 R, float32 quats[4R], float32 weights[R] to the file argv[2].
 * The reference also writes debug_samples.data into the working directory,
 * so callers run this from a scratch directory.  Test infrastructure. */
#include <stdio.h>
#include <stdlib.h>
#include "rotations.h"

int main(int argc, char** argv) {
  if (argc != 3) {
    fprintf(stderr, "usage: %s n out.bin\n", argv[0]);
    return 2;
  }
  const int n = atoi(argv[1]);
  Quaternion** list = NULL;
  real* weights = NULL;
  const int R = generate_rotation_list(n, &list, &weights);
  FILE* f = fopen(argv[2], "wb");
  if (!f) return 3;
  fwrite(&R, sizeof(int), 1, f);
  for (int i = 0; i < R; ++i) fwrite(list[i]->q, sizeof(real), 4, f);
  fwrite(weights, sizeof(real), (size_t)R, f);
  fclose(f);
  return 0;
}
