/* gsplat.h -- C ABI of the GB300 Gaussian-splatting rasterizer (libmpm.so).
 *
 * The differentiable tile rasterizer that consumes the simulated particles
 * in the reference's end-to-end mode (renderer/core/renderer.py:347-510 via
 * the diff_gauss module): per-Gaussian projection, tile binning by
 * (tile, depth), front-to-back alpha blending of color, depth, normal, alpha
 * and extra channels, and the exact adjoint of all of it.  It replaces
 *   - _C.rasterize_gaussians          rasterize_points.cu:35-132
 *   - _C.rasterize_gaussians_backward rasterize_points.cu:135-238
 * whose work is rasterizer_impl.cu:54-116 (binning), forward.cu:204-455
 * (preprocess, render) and backward.cu:144-700 (render and preprocess
 * adjoints).  The Python module diff_gauss (this repository) calls these
 * entry points with device pointers from torch tensors.
 *
 * All pointers are device pointers, float32 unless stated, row-major.  A
 * frame runs as gs_preprocess (per Gaussian; returns how many (tile,
 * Gaussian) pairs the frame renders), then gs_render, then on demand
 * gs_backward.  The caller owns every buffer (see GsGeom, GsBinning,
 * GsImage) and sizes the two scratch buffers with gs_scratch_bytes.
 * Every function returns an MPM_* status (mpm.h); mpm_last_error() holds
 * the message.
 */
#ifndef GSPLAT_H
#define GSPLAT_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GS_TILE 16         /* tile = 16 x 16 pixels, one CUDA block */
#define GS_MAX_EXTRA 34    /* extra blended channels (diff_gauss limit) */

/* the scene and the camera (GaussianRasterizationSettings + inputs) */
typedef struct GsScene {
    int P;                      /* Gaussians */
    int H, W;                   /* image */
    float tanfovx, tanfovy, scale_modifier;
    int sh_degree, sh_coeffs;   /* active SH degree; coefficients per Gaussian in shs (0: no SH) */
    int extra_dims;             /* channels of extra (0..GS_MAX_EXTRA) */
    const float* bg;            /* (3) */
    const float* viewmatrix;    /* (16): x' = m[0]x + m[4]y + m[8]z + m[12] (rasterizer convention) */
    const float* projmatrix;    /* (16), same convention, homogeneous */
    const float* campos;        /* (3) */
    const float* means3D;       /* (P,3) */
    const float* opacities;     /* (P) */
    const float* shs;           /* (P,sh_coeffs,3) or NULL */
    const float* colors;        /* (P,3) precomputed colors or NULL (then shs) */
    const float* scales;        /* (P,3) or NULL */
    const float* rotations;     /* (P,4) quaternion (w,x,y,z), used as given, or NULL */
    const float* cov3D;         /* (P,6) precomputed (xx,xy,xz,yy,yz,zz) or NULL (then scales/rotations) */
    const float* norm3D;        /* (P,3) precomputed normals or NULL (then from scales/rotations) */
    const float* extra;         /* (P,extra_dims) or NULL */
    /* 0: the reference's gradients (the default of the Python module): the
     * rotation gradient through a normal taken from scales/rotations carries
     * the sign backward.cu:364-366 gives it, which tests a row of the
     * rotation matrix where the forward pass took a column (forward.cu:188),
     * so for some Gaussians it is the negated derivative; 1: the exact
     * derivative of the forward pass.  Everything else is the same. */
    int exact_adjoint;
} GsScene;

/* per-Gaussian results of gs_preprocess (caller-allocated, P entries each) */
typedef struct GsGeom {
    int* radii;                 /* (P) int32, 0 = culled */
    float* xy;                  /* (P,2) pixel-space mean */
    float* depth;               /* (P) view-space z */
    float* conic_opacity;       /* (P,4) inverse 2D covariance (a,b,c) and opacity */
    float* rgb;                 /* (P,3) color (from SH or precomputed) */
    float* normal;              /* (P,3) */
    float* cov3D;               /* (P,6) world covariance used */
    uint8_t* clamped;           /* (P,3) SH color clamped at 0 */
    uint32_t* tiles_touched;    /* (P) */
    uint32_t* offsets;          /* (P) inclusive prefix sum of tiles_touched */
} GsGeom;

/* (tile, Gaussian) pairs of one frame (caller-allocated; L = num_rendered) */
typedef struct GsBinning {
    uint64_t* keys;             /* (L) */
    uint64_t* keys_sorted;      /* (L) */
    uint32_t* ids;              /* (L) */
    uint32_t* ids_sorted;       /* (L): Gaussian per sorted pair (tile, then depth) */
    uint32_t* ranges;           /* (tiles,2): [start,end) of each tile in ids_sorted */
} GsBinning;

/* rendered frame (caller-allocated) */
typedef struct GsImage {
    float* color;               /* (3,H,W) */
    float* depth;               /* (1,H,W) */
    float* normal;              /* (3,H,W), not normalised */
    float* alpha;               /* (1,H,W) = 1 - final transmittance */
    float* extra;               /* (extra_dims,H,W) or NULL */
    uint32_t* n_contrib;        /* (H,W): index+1 of the last blended pair of the pixel's tile list */
} GsImage;

/* gradients out of gs_backward (caller-allocated, zeroed by gs_backward) */
typedef struct GsGrads {
    float* means3D;             /* (P,3) */
    float* means2D;             /* (P,3): dL/d(projected mean) in NDC units, third entry 0 */
    float* opacities;           /* (P) */
    float* colors;              /* (P,3): dL/dcolor (precomputed colors, or the SH color) */
    float* shs;                 /* (P,sh_coeffs,3) or NULL */
    float* scales;              /* (P,3) or NULL */
    float* rotations;           /* (P,4) or NULL */
    float* cov3D;               /* (P,6): dL/d(cov3D entries) */
    float* norm3D;              /* (P,3) */
    float* extra;               /* (P,extra_dims) or NULL */
    float* conic;               /* (P,3) scratch: dL/d(conic a,b,c) */
    float* depth;               /* (P) scratch: dL/d(view depth) */
} GsGrads;

/* scratch of the prefix sum over P entries and of the radix sort of L pairs */
int gs_scratch_bytes(int P, int L, int tiles, size_t* scan_bytes, size_t* sort_bytes);
/* forward.cu:204-318 + rasterizer_impl.cu prefix sum: *num_rendered = total
 * tile overlaps (the one host synchronisation of a frame) */
int gs_preprocess(const GsScene* s, const GsGeom* g, void* scan_tmp, size_t scan_bytes, int* num_rendered,
                  void* stream);
/* rasterizer_impl.cu:54-116 binning + forward.cu:321-455 blending */
int gs_render(const GsScene* s, const GsGeom* g, int num_rendered, const GsBinning* b, void* sort_tmp,
              size_t sort_bytes, const GsImage* img, void* stream);
/* backward.cu: adjoint of gs_render and gs_preprocess.  The dL_d* inputs
 * match the GsImage outputs (any may be NULL = zero). */
int gs_backward(const GsScene* s, const GsGeom* g, int num_rendered, const GsBinning* b, const GsImage* img,
                const float* dL_dcolor, const float* dL_ddepth, const float* dL_dnormal, const float* dL_dalpha,
                const float* dL_dextra, const GsGrads* out, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* GSPLAT_H */
