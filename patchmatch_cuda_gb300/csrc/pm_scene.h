/*
 * pm_scene.h -- seeded synthetic multi-view scenes for PatchMatch MVS.
 *
 * A scene is a set of textured planes and boxes in world space. Cameras orbit a pivot
 * point on the world z axis; rendering ray-casts every pixel centre (x + 1/2, y + 1/2)
 * and returns an 8-bit grayscale image plus the z-depth of the visible surface in that
 * camera (the depth the PatchMatch engine estimates). Texture is value noise in each
 * surface's own coordinates, so it is consistent across views.
 *
 * Camera convention (Middlebury par files): x_cam = R X + t, pixel ~ K x_cam, image x
 * right, y down, z forward.
 */
#ifndef PM_SCENE_H
#define PM_SCENE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct pm_scene pm_scene;

/* Creates a scene of n_planes slanted planes and n_boxes rotated boxes, placed so that
 * a camera at yaw = pitch = 0 (at the world origin, looking down +z, focal length
 * `focal` for a `width`-wide image) sees depths inside [depth_near, depth_far].
 * Returns NULL on invalid arguments. */
pm_scene *pm_scene_create(uint64_t seed, int n_planes, int n_boxes, double depth_near,
                          double depth_far, int width, int height, double focal);
void pm_scene_destroy(pm_scene *scene);

/* Orbit camera: looks at the pivot (0, 0, z_pivot) from distance z_pivot, rotated by yaw
 * (about the y axis) and pitch (about the camera x axis), degrees. Principal point at the
 * image centre (width/2, height/2). */
void pm_scene_camera(const pm_scene *scene, double yaw_deg, double pitch_deg, int width,
                     int height, double focal, double K[9], double R[9], double t[3]);

/* Renders one view. image: height*width u8; depth: height*width float z-depth (may be
 * NULL). Returns the number of pixels whose ray hit nothing (rendered 0, depth 0). */
int pm_scene_render(const pm_scene *scene, const double K[9], const double R[9],
                    const double t[3], int width, int height, uint8_t *image, float *depth);

double pm_scene_pivot_depth(const pm_scene *scene);

#ifdef __cplusplus
}
#endif
#endif
