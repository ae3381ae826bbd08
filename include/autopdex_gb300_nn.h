/*
 * autopdex_gb300 -- BF16 tensor-core kernels of the learned preconditioner.
 *
 * No counterpart in AutoPDEx: these kernels implement the convolutional network that
 * this backend applies inside flexible CG ('type of preconditioner': 'learned').  Tensors
 * are NHWC bf16 device arrays; every function launches on `stream` and returns 0 or a
 * negative status (AGX_ERR_ARG, AGX_ERR_UNSUPPORTED, AGX_ERR_CUDA).  `err` (device int)
 * is set to 1 by a CTA whose tensor-core work did not complete within its wait limit.
 */
#ifndef AUTOPDEX_GB300_NN_H
#define AUTOPDEX_GB300_NN_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* out = act(conv3x3(concat(in1[c1], in2[c2])) + bias), cout output channels written as
   out1 (channels [0, split)) and out2 (channels [split, cout)); relu: 0 or 1, plus
   AGX_NN_CONST_WEIGHTS when wpk and bias were not written by the kernel launched just before
   this one on the stream (their copy then overlaps that kernel's tail), plus AGX_NN_LOADER(l)
   to choose this launch's halo loader (l as agx_nn_set_halo_loader, 0 .. 2; without it the
   process-wide choice applies).  Packed weights from agx_nn_pack_weights (mode 0), or the
   input-gradient image (mode 1) with in1 = output gradient, no bias and relu = 0. */
#define AGX_NN_CONST_WEIGHTS 2
#define AGX_NN_LOADER(l) (((l) + 1) << 4)
int agx_nn_conv3x3(const void* in1, const void* in2, int c1, int c2, const void* wpk, const float* bias,
                   void* out1, void* out2, int split, int cout, int relu, int B, int H, int W, int* err,
                   void* stream);
/* How agx_nn_conv3x3 feeds its tensor cores: 0 cp.async halo copies by all threads of the CTA
   (16-byte pixel chunks, zero fill at the image edge; in1 and in2 then 16-byte aligned) and one
   loop with a CTA barrier per tile; 1 one tensor-memory-access copy per 8-channel plane in the
   same loop; 2 the tensor copies in a warp-specialised kernel (a copy warp, an MMA warp and four
   epilogue warps on mbarrier rings); 3 (the default) 2 for two-input layers of at least 128^2
   pixels, else 1.  All give identical results.  Process-wide; affects later launches only. */
int agx_nn_set_halo_loader(int loader);
/* A device int that the inference kernels launched from now on (convolutions, pooling,
   upsampling, the grid transfers and images) read after waiting for their predecessor: nonzero
   makes them return at once.  A preconditioner passes the solve's converged flag
   (agx_solve_flag), so that iterations a captured CUDA-graph chunk runs past convergence skip
   the network; NULL (the default) turns it off.  Process-wide; launches keep the pointer they
   were given, graph captures included. */
int agx_nn_set_skip_flag(const int* flag);
/* dw_rows[(tap * (c1 + c2) + ci) * cout + co] += sum over pixels of in(p + tap)[ci] * dout(p)[co] */
int agx_nn_wgrad3x3(const void* in1, const void* in2, int c1, int c2, const void* dout, int cout, float* dw_rows,
                    int B, int H, int W, int* err, void* stream);
/* f32 weights [cout][cin][3][3] -> bf16 operand image; mode 0 forward, 1 input gradient */
int agx_nn_pack_weights(const float* w, int cout, int cin, int mode, void* img, void* stream);
/* wgrad rows -> f32 [cout][cin][3][3] */
int agx_nn_unpack_wgrad(const float* dw_rows, int cout, int cin, float* dw, void* stream);
/* 2x2 average pooling (backward = 0) or its adjoint (backward = 1); H, W: full size */
int agx_nn_pool2(const void* in, void* out, int B, int H, int W, int C, int backward, void* stream);
/* nearest 2x upsampling (backward = 0) or its adjoint; H, W: coarse size */
int agx_nn_upsample2(const void* in, void* out, int B, int H, int W, int C, int backward, void* stream);
/* f x f average pooling (backward = 0: out = block means) or its adjoint (backward = 1: every
   pixel of a block gets the coarse value / f^2); H, W: full size, multiples of f.  C a multiple
   of 8, in and out 16-byte aligned; sums in float, rounded to bf16 once. */
int agx_nn_pool(const void* in, void* out, int B, int H, int W, int C, int f, int backward, void* stream);
/* nearest f x upsampling (backward = 0) or its adjoint (backward = 1: block sums); H, W: coarse
   size.  Same channel and alignment rules as agx_nn_pool. */
int agx_nn_upsample(const void* in, void* out, int B, int H, int W, int C, int f, int backward, void* stream);
/* g *= (y > 0) */
int agx_nn_relu_backward(void* g, const void* y, int64_t n, void* stream);
/* a += b */
int agx_nn_add(void* a, const void* b, int64_t n, void* stream);
/* db[c] += sum over P pixels of g[p][c] */
int agx_nn_bias_grad(const void* g, int64_t P, int C, float* db, void* stream);
/* node vector (Hn x Wn, node i*Wn + j) -> NHWC 16-channel image Hp x Wp: channel 0 the
   vector (scaled to unit rms when normalize; 1/rms written to scale[0]), channel 1 aux */
int agx_nn_grid_from_vector(const float* r, const float* aux, int Hn, int Wn, int Hp, int Wp, int normalize,
                            float* scale, void* img, void* stream);
/* Bilinear grid transfer for a network applied on a coarser node grid.  The fine grid has
   ((Hc - 1) f + 1) x ((Wc - 1) f + 1) nodes (node i*Wf + j) and its node (f I, f J) is coarse
   node (I, J).  agx_nn_prolong: fine = P coarse, P the bilinear interpolation;
   agx_nn_restrict: coarse = P^T fine, with coarse nodes whose fine node is flagged in
   `fixed` (optional, one byte per fine node: the Dirichlet nodes) set to zero. */
int agx_nn_restrict(const float* fine, const unsigned char* fixed, int Hc, int Wc, int f, float* coarse,
                    void* stream);
int agx_nn_prolong(const float* coarse, int Hc, int Wc, int f, float* fine, void* stream);
/* channel 0 of an NHWC image with C channels -> node vector */
int agx_nn_vector_from_grid(const void* img, int C, int Hn, int Wn, int Wp, float* z, void* stream);
/* The same transfers for a node field of nd (1 .. 3) components stored node-major
   (r[node nd + c], the DOF numbering of an (n_nodes, nd) array): agx_nn_grid_from_field writes
   channels 0 .. nd-1 (scaled to unit rms over all components when normalize) and naux
   per-node features aux[node naux + a] into channels nd .. nd+naux-1 (nd + naux <= 16);
   agx_nn_field_from_grid reads channels 0 .. nd-1; agx_nn_restrict_field /
   agx_nn_prolong_field transfer every component bilinearly, `fixed` flagging fine DOFs. */
int agx_nn_grid_from_field(const float* r, int nd, const float* aux, int naux, int Hn, int Wn, int Hp, int Wp,
                           int normalize, float* scale, void* img, void* stream);
int agx_nn_field_from_grid(const void* img, int C, int nd, int Hn, int Wn, int Wp, float* z, void* stream);
int agx_nn_restrict_field(const float* fine, const unsigned char* fixed, int nd, int Hc, int Wc, int f, float* coarse,
                          void* stream);
int agx_nn_prolong_field(const float* coarse, int nd, int Hc, int Wc, int f, float* fine, void* stream);
/* The coarse-grid network's transfers in fewer launches.  agx_nn_restrict_image: coarse =
   P^T fine (as agx_nn_restrict_field) and the network's input image of (coarse / rms, aux) with
   1 / rms in scale[0] (as agx_nn_grid_from_field with normalize = 1) in two launches: the
   restriction leaves per-block sums of squares in `work` (agx_nn_restrict_image_work() doubles)
   and every block of the image kernel adds them up itself.  agx_nn_prolong_image: fine = P
   applied to channels 0 .. nd-1 of an NHWC image with C channels (the network's output; the
   coarse field is not written out), zero at the DOFs flagged in `fixed` (optional).  Grids
   below 2^31 entries; the fine grid at most 65535 rows. */
int agx_nn_restrict_image_work(void);
int agx_nn_restrict_image(const float* fine, const unsigned char* fixed, int nd, const float* aux, int naux, int Hc,
                          int Wc, int f, int Hp, int Wp, float* coarse, double* work, float* scale, void* img,
                          void* stream);
int agx_nn_prolong_image(const void* img, int C, int nd, int Hc, int Wc, int Wp, int f, const unsigned char* fixed,
                         float* fine, void* stream);

/* ---- the 3-D network (structured brick meshes) -----------------------------------------
   Tensors are NDHWC bf16 (batch, z, y, x, channel).  agx_nn_conv3x3x3: 3x3x3 convolution,
   stride 1, zero padding 1, of concat(in1 [c1 channels], in2 [c2]) with the weight image of
   agx_nn_pack_weights3d (mode 0: forward; mode 1: the input-gradient image, whose output
   splits into out1 [split channels] and out2 [cout - split]); relu as agx_nn_conv3x3
   (bit 0 ReLU, AGX_NN_CONST_WEIGHTS).  Supported (c1, c2, cout): (16, 0, 16) with and without
   ReLU, (16, 16, 16) with ReLU, (16, 0, 32) without (the input gradient of a concatenating
   layer).  Tensors 16-byte aligned.  agx_nn_wgrad3x3x3 accumulates dW rows (27 (c1 + c2)) x cout
   as agx_nn_wgrad3x3 does, for (16, 0, 16) and (16, 16, 16); agx_nn_unpack_wgrad3d turns them
   into the [cout][cin][3][3][3] layout.  Taps are t = 9 dz + 3 dy + dx. */
int agx_nn_conv3x3x3(const void* in1, const void* in2, int c1, int c2, const void* wpk, const float* bias, void* out1,
                     void* out2, int split, int cout, int relu, int B, int D, int H, int W, int* err, void* stream);
int agx_nn_wgrad3x3x3(const void* in1, const void* in2, int c1, int c2, const void* dout, int cout, float* dw_rows,
                      int B, int D, int H, int W, int* err, void* stream);
int agx_nn_pack_weights3d(const float* w, int cout, int cin, int mode, void* img, void* stream);
int agx_nn_unpack_wgrad3d(const float* dw_rows, int cout, int cin, float* dw, void* stream);
/* f x f x f average pooling (backward = 0; D, H, W: full size, multiples of f) or its adjoint
   (backward = 1: every voxel of a block gets coarse / f^3); nearest f x upsampling (backward = 0;
   D, H, W: coarse size) or its adjoint (block sums).  C a multiple of 8, 16-byte aligned. */
int agx_nn_pool3d(const void* in, void* out, int B, int D, int H, int W, int C, int f, int backward, void* stream);
int agx_nn_upsample3d(const void* in, void* out, int B, int D, int H, int W, int C, int f, int backward, void* stream);
/* Transfers between the scalar node field of a structured brick mesh -- ((Dc-1) f + 1) x
   ((Hc-1) f + 1) x ((Wc-1) f + 1) nodes, node (i, j, k) at (i Hf + j) Wf + k -- and the
   network's coarse grid of Dc x Hc x Wc nodes, coarse node (I, J, K) on fine node (f I, f J, f K);
   P is trilinear interpolation.  agx_nn_restrict_image3d: coarse = P^T fine (zero where the
   fine node under it is flagged in `fixed`, optional) and the input image (Dp x Hp x Wp voxels,
   16 channels: coarse / rms, then 1 inside the coarse grid) with 1 / rms in scale[0], in two
   launches (`work`: agx_nn_restrict_image3d_work() doubles).  agx_nn_restrict3d: coarse = P^T
   fine alone.  agx_nn_prolong_image3d: fine = P applied to channel 0 of an image with C
   channels, zero at flagged nodes. */
int agx_nn_restrict_image3d_work(void);
int agx_nn_restrict_image3d(const float* fine, const unsigned char* fixed, int Dc, int Hc, int Wc, int f, int Dp,
                            int Hp, int Wp, float* coarse, double* work, float* scale, void* img, void* stream);
int agx_nn_restrict3d(const float* fine, const unsigned char* fixed, int Dc, int Hc, int Wc, int f, float* coarse,
                      void* stream);
int agx_nn_prolong_image3d(const void* img, int C, int Dc, int Hc, int Wc, int Hp, int Wp, int f,
                           const unsigned char* fixed, float* fine, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* AUTOPDEX_GB300_NN_H */
