/* libbsc's BWT-stage entry points forwarded to the GB300 block sorter (see
 * include/qzgpu_bsc_shim.h).  Plain C, built separately from libqzgpu.so so
 * that only a caller who wants libbsc's own symbols replaced links it. */
#include "qzgpu.h"
#include "qzgpu_bsc_shim.h"

/* The GPU codes past libbsc's GPU range fold into the nearest libbsc code. */
static int to_libbsc(int rc) {
    if (rc == QZGPU_TIMEOUT) return QZGPU_GPU_ERROR;
    if (rc == QZGPU_BLOCK_TOO_LARGE) return QZGPU_BAD_PARAMETER;
    return rc;
}

int bsc_bwt_encode(unsigned char *T, int n, unsigned char *num_indexes, int *indexes, int features) {
    return to_libbsc(qzgpu_bwt_encode(T, n, num_indexes, indexes, features));
}

int bsc_bwt_decode(unsigned char *T, int n, int index, unsigned char num_indexes, int *indexes, int features) {
    return to_libbsc(qzgpu_bwt_decode(T, n, index, num_indexes, indexes, features));
}
