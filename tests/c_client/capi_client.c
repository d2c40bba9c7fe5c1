/* A plain C99 client of include/rrtl_cuda.h: links librrtl_gb300.so and makes
 * the host-only calls (no device needed). argv[1] is a design JSON file whose
 * top module is argv[2]. Exits 0 when every check holds. */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "rrtl_cuda.h"

static int fail(const char* what) {
  fprintf(stderr, "FAIL %s: %s\n", what, rrtl_last_error());
  return 1;
}

int main(int argc, char** argv) {
  if (argc != 3) return 2;
  FILE* f = fopen(argv[1], "rb");
  if (!f) return 2;
  fseek(f, 0, SEEK_END);
  long n = ftell(f);
  fseek(f, 0, SEEK_SET);
  char* json = malloc((size_t)n + 1);
  if (!json || fread(json, 1, (size_t)n, f) != (size_t)n) return 2;
  json[n] = 0;
  fclose(f);

  rrtl_ctx* ctx = NULL;
  if (rrtl_ctx_create(0, NULL) != RRTL_E_ARG) return fail("ctx_create(NULL out)");
  if (strncmp(rrtl_last_error(), "E_ARG", 5) != 0) return fail("last_error code");
  (void)ctx;

  /* bit-slice plane design: size query, then the text */
  size_t len = 0;
  if (rrtl_bitslice_json(json, (size_t)n, argv[2], NULL, 0, &len) != RRTL_OK || len == 0) return fail("bitslice size");
  char* planes = malloc(len + 1);
  if (rrtl_bitslice_json(json, (size_t)n, argv[2], planes, len + 1, &len) != RRTL_OK) return fail("bitslice text");
  if (strstr(planes, "[0]") == NULL) return fail("plane names");

  /* compiled word kernel source for the general run, no compile */
  size_t src_len = 0;
  uint32_t cubin = 0;
  if (rrtl_word_jit_emit(json, (size_t)n, argv[2], NULL, NULL, NULL, 0, &src_len, &cubin, NULL, 0, 0) != RRTL_OK ||
      src_len == 0 || cubin != 0)
    return fail("word_jit_emit size");
  char* src = malloc(src_len + 1);
  if (rrtl_word_jit_emit(json, (size_t)n, argv[2], NULL, NULL, src, src_len + 1, &src_len, &cubin, NULL, 0, 0) !=
      RRTL_OK)
    return fail("word_jit_emit text");
  if (strstr(src, "rrtl_word_jit") == NULL) return fail("kernel name in source");

  /* a single module does not fold: an error code with the reference's diagnostic */
  char plan[256];
  size_t plan_len = 0;
  if (rrtl_instance_fold_plan(json, (size_t)n, argv[2], plan, sizeof plan, &plan_len) != RRTL_E_UNSUPPORTED)
    return fail("instance_fold_plan of a leaf module");
  if (strstr(rrtl_last_error(), "E_INSTANCE_FOLD") == NULL) return fail("fold diagnostic");

  free(src);
  free(planes);
  free(json);
  printf("c client ok\n");
  return 0;
}
