// Seeded synthetic RGB-D sequence generator (host code, C ABI).
#ifndef SF_SYNTH_H_
#define SF_SYNTH_H_
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { SF_SCENE_ROOM = 0, SF_SCENE_CORRIDOR = 1 };
enum { SF_TRAJ_CIRCLE = 0, SF_TRAJ_SPLINE = 1, SF_TRAJ_FORWARD = 2 };

typedef struct {
  int scene;          /* SF_SCENE_*                                       */
  int trajectory;     /* SF_TRAJ_*                                        */
  int cols, rows;
  float fx, fy, cx, cy;
  float depth_scale;  /* depth units per metre (1000 = mm)                */
  float dropout;      /* fraction of depth pixels set to 0                */
  float label_flip;   /* fraction of mask pixels replaced by a random id  */
  int n_objects;      /* primitives (0 = scene default)                   */
  float noise;        /* multiplier on the depth-noise sigma (1 = model)  */
  uint64_t seed;
} sf_synth_config;

typedef struct sf_synth sf_synth;

int sf_synth_create(const sf_synth_config *cfg, sf_synth **out);
int sf_synth_destroy(sf_synth *s);
/* Ground-truth camera->world pose of frame i, row-major 4x4. */
int sf_synth_pose(const sf_synth *s, int i, double *pose16);
/* Renders frame i: depth uint16[rows*cols], rgb uint8[rows*cols*3],
 * mask uint8[rows*cols] (any may be NULL), pose16 (may be NULL). */
int sf_synth_frame(const sf_synth *s, int i, uint16_t *depth, uint8_t *rgb,
                   uint8_t *mask, double *pose16);

#ifdef __cplusplus
}
#endif
#endif
