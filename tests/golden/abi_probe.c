/* Prints the layout of rawspec_context as JSON.  Compiled against the
 * reference header (to make the fixture) and against include/rawspec.h (in
 * the tests); the two outputs must be identical. */
#include <stddef.h>
#include <stdio.h>
#include "rawspec.h"

#define F(m) printf("  \"%s\": [%zu, %zu],\n", #m, offsetof(rawspec_context, m), sizeof(((rawspec_context *)0)->m))

int main(void) {
  printf("{\n");
  F(No); F(Np); F(Nant); F(Nc); F(Ntpb); F(exit_soon); F(Nbc); F(Nbps); F(Npolout); F(Nts); F(Nas);
  F(dump_callback); F(user_data); F(Nb); F(Nb_host); F(h_blkbufs); F(gpu_index); F(input_conjugated);
  F(incoherently_sum); F(Naws); F(Aws); F(h_pwrbuf); F(h_pwrbuf_size); F(h_icsbuf); F(Nds); F(Ntmax); F(gpu_ctx);
  printf("  \"MAX_OUTPUTS\": [%d, 0],\n", MAX_OUTPUTS);
  printf("  \"RAWSPEC_FORWARD_FFT\": [%d, 0],\n", RAWSPEC_FORWARD_FFT);
  printf("  \"RAWSPEC_INVERSE_FFT\": [%d, 0],\n", RAWSPEC_INVERSE_FFT);
  printf("  \"RAWSPEC_CALLBACK_PRE_DUMP\": [%d, 0],\n", RAWSPEC_CALLBACK_PRE_DUMP);
  printf("  \"RAWSPEC_CALLBACK_POST_DUMP\": [%d, 0],\n", RAWSPEC_CALLBACK_POST_DUMP);
  printf("  \"RAWSPEC_FILE\": [%d, 0],\n", (int)RAWSPEC_FILE);
  printf("  \"RAWSPEC_NET\": [%d, 0],\n", (int)RAWSPEC_NET);
  printf("  \"sizeof\": [%zu, 0]\n}\n", sizeof(rawspec_context));
  return 0;
}
