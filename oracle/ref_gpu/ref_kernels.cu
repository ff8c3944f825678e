/*
 * TEST INFRASTRUCTURE ONLY — compiled by oracle/Makefile ("make refgpu") into
 * device-only cubins under oracle/_ref/.
 *
 * Includes the reference's own CUDA sources IN PLACE from the reference tree
 * (include path set by the Makefile; nothing is copied):
 *   src/stabilization/flowconsistency.cu   kernel_warp, kernel_adap_comb,
 *       kernel_consist_wt, kernel_consist_out, kernel_bilinear
 *   src/stabilization/gpuimage.cu          kernel_to_float_image, kernel_to_char_image
 *   src/ort_custom_ops/src/opticalflow/correlation_cuda.cu, warp_cuda.cu
 * The cubins are loaded on the GPU by oracle/ref_gpu/ref_gpu_harness.cu to
 * run the reference's kernels with the reference's launch geometry.
 */
#include "flowconsistency.cu"
#include "gpuimage.cu"
#include "correlation_cuda.cu"
#include "warp_cuda.cu"
