/* Seeded synthetic depth sequences (host C++, see synth.cpp). */
#pragma once
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
  int width, height;
  float fx, fy, cx, cy;
  int n_frames;
  uint64_t seed;
  double orbit_radius;     /* horizontal orbit radius (m)                   */
  double view_distance;    /* camera distance to the scene centre (m)       */
  double orbit_start_deg;  /* azimuth of frame 0                            */
  double orbit_step_deg;   /* azimuth step per frame                        */
  double jitter_deg;       /* Gaussian jitter of azimuth and roll (deg)     */
  double jitter_m;         /* Gaussian jitter of position and target (m)    */
  int noise;               /* 1 = axial noise on                            */
  double dropout_iid;      /* fraction of pixels dropped independently      */
  double dropout_blob;     /* fraction of pixels dropped in 8x8 blobs       */
  double max_depth;        /* depths beyond this become 0 (0 = no cut-off)  */
  int threads;             /* 0 = all host threads                          */
} vs_synth_config;

void vs_synth_default(vs_synth_config* c, int width, int height);
/* depth: n_frames*height*width uint16 (mm).  T_gc: n_frames*16 ground-truth
 * poses (global = camera 0, row-major).  centre_cam0: scene centre in the
 * global frame (3).  T_gc / centre_cam0 may be NULL.  Returns 0 on success. */
int vs_synth_generate(const vs_synth_config* c, uint16_t* depth, double* T_gc,
                      double* centre_cam0);
/* the same plus a registered colour image per frame: rgb is
 * n_frames * 3 * height * width uint8, planar R, G, B per frame (a smooth
 * texture of the true surface point; 0 where the ray hits nothing) */
int vs_synth_generate_rgb(const vs_synth_config* c, uint16_t* depth, uint8_t* rgb, double* T_gc,
                          double* centre_cam0);

#ifdef __cplusplus
}
#endif
