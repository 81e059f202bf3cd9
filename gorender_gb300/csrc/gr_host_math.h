// gr_host_math.h -- host restatement of matrix.go / vector.go / mesh.go.
#pragma once

namespace gr {

void mat_identity(float* m);
void mat_multiply(const float* a, const float* b, float* out);
void world_matrix(const float* scale, const float* rot, const float* trans, float* out);
void view_matrix(const float* eye, const float* dir, const float* up, float* out);
void perspective_matrix(float fov, float aspect, float znear, float zfar, float* out);
void screen_matrix(int width, int height, float* out);
void object_matrices(const float* scale, const float* rot, const float* trans, const float* eye,
                     const float* dir, const float* up, int width, int height, float fov_y,
                     float* mvp, float* world);
void normalize3(const float* v, float* out);
void face_normals(const float* pos, const int* vidx, int nf, float* out);
void bounding_box(const float* pos, int nv, float* out);

}  // namespace gr
