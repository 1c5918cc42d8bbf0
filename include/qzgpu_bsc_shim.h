/*
 * libbsc BWT-stage symbols backed by the GB300 block sorter (optional shim).
 *
 * qz links libbsc statically and reaches its block-sorting stage only through
 * bsc_compress / bsc_decompress (crates/qz-lib/src/compression/bsc.rs:91-125,
 * library named at bsc.rs:91; built by crates/qz-lib/build.rs:56-75 and, with
 * the cuda feature, build.rs:179-224).  Inside libbsc those two calls run the
 * BWT stage through bsc_bwt_encode / bsc_bwt_decode (libbsc/bwt/bwt.h, not in
 * the reference tree).  The object built from qz_gb300/csrc/bsc_bwt_shim.c
 * (qz_gb300/_lib/bsc_bwt_shim.o, linked together with libqzgpu.so) exports
 * those two symbols, so a libbsc built without its own bwt object links
 * against the GPU sorter and qz's Rust code changes not at all.
 *
 * Codes: 0 and libbsc's -1..-6 as qzgpu returns them; the GPU codes -7..-9
 * (GPU error, no usable GPU, not enough GPU memory) keep their numbers, and
 * -10 (timed out) and -11 (block too large) fold into -7 and -1, so a caller
 * sees only -1..-9.  C linkage.
 */
#ifndef QZGPU_BSC_SHIM_H
#define QZGPU_BSC_SHIM_H

#ifdef __cplusplus
extern "C" {
#endif

/* libbsc's forward BWT stage, run by bsc_compress for blockSorter = BWT
 * (called at bsc.rs:172-183): T[0..n) transformed in place; returns the
 * primary index or a negative code; auxiliary indexes as qzgpu_bwt_encode. */
int bsc_bwt_encode(unsigned char *T, int n, unsigned char *num_indexes, int *indexes, int features);

/* libbsc's inverse BWT stage, run by bsc_decompress after the QLFC decoder
 * (called at bsc.rs:421-433): T[0..n) holds the BWT and receives the block. */
int bsc_bwt_decode(unsigned char *T, int n, int index, unsigned char num_indexes, int *indexes, int features);

#ifdef __cplusplus
}
#endif

#endif /* QZGPU_BSC_SHIM_H */
