/*
 * gorender_diff.c -- FP64 restatement of the differentiable shading model.
 *
 * TEST INFRASTRUCTURE ONLY (the checker of the CUDA differentiable path; see
 * gorender_oracle.h).  The model is an extension with no counterpart in the
 * reference renderer; it is shaded over fixed visibility (the face the
 * reference raster leaves at each pixel) and is written out here as plainly
 * as possible, in double precision, with its hand-derived adjoint:
 *
 *   clip_k = MVP p_k,  s_k = S (clip_k / W_k)          (k = 0, 1, 2: face corners)
 *   e_0 = (x1-x)(y2-y) - (x2-x)(y1-y), e_1, e_2 cyclic  at pixel (x, y)
 *   r_k = e_k / W_k,  b_k = r_k / (r_0 + r_1 + r_2)
 *   l_k = max(b_k, 0) / sum_j max(b_j, 0)             (clipped to the face)
 *   c = sum l_k c_k,  I = sum l_k I_k,  I_k = 0.5 + 0.5 nhat_k . L
 *   nhat_k = xyz of Vec4.Normalize(world * n_k)         (renderer.go:328-331)
 *   t = tex[floor(v th) mod th][floor(u tw) mod tw],  (u, v) = sum l_k uv_k
 *   out = (I c_r t_r, I c_g t_g, I c_b t_b, t_a),  loss = sum (out - target)^2
 */
#include <math.h>
#include <stddef.h>
#include <stdint.h>
#include <string.h>

#include "gorender_oracle.h"

#define NO_FACE 0xFFFFFFFFu

static void mat4_apply(const double* m, const double* v, double* r) {
  for (int i = 0; i < 4; i++) r[i] = m[4 * i] * v[0] + m[4 * i + 1] * v[1] + m[4 * i + 2] * v[2] + m[4 * i + 3] * v[3];
}

static int wrap_index(double u, int n) {
  double f = floor(u * (double)n);
  if (!(f > -2.0e9 && f < 2.0e9)) return 0;
  int i = (int)f % n;
  return i < 0 ? i + n : i;
}

double orc_diff_eval(const orc_diff_scene* s, const orc_diff_view* views, int32_t nviews, const uint32_t* ids,
                     const uint32_t* texel_in, uint32_t* texel_out, const float* target, double* image,
                     double* g_pos, double* g_vcol, double* g_tex, double* g_light) {
  if (g_pos) memset(g_pos, 0, sizeof(double) * 4 * (size_t)s->nv);
  if (g_vcol) memset(g_vcol, 0, sizeof(double) * 3 * (size_t)s->nv);
  if (g_tex && s->tex) memset(g_tex, 0, sizeof(double) * 4 * (size_t)s->tw * (size_t)s->th);
  if (g_light) g_light[0] = g_light[1] = g_light[2] = 0.0;
  double loss = 0.0;
  size_t base = 0;
  for (int32_t v = 0; v < nviews; v++) {
    const orc_diff_view* vw = &views[v];
    const size_t npx = (size_t)vw->width * (size_t)vw->height;
    for (size_t p = 0; p < npx; p++) {
      const size_t gp = base + p;
      const double px = (double)(p % (size_t)vw->width), py = (double)(p / (size_t)vw->width);
      const float* tg = target + 4 * gp;
      double out[4] = {0, 0, 0, 0};
      uint32_t texel = NO_FACE;
      const uint32_t id = ids[gp];
      int shaded = 0;
      int vi[3] = {0, 0, 0}, ni[3] = {0, 0, 0};
      double clip[3][4], sx[3], sy[3], e[3], r[3], R = 0, b[3], l[3], msum = 1, Ik[3], nh[3][3];
      double col[3] = {0, 0, 0}, I = 0;
      double t[4] = {1, 1, 1, 1};
      int32_t f = -1;
      if (id != NO_FACE) {
        f = (int32_t)(id - (uint32_t)v * (uint32_t)s->nf);
        int ok = f >= 0 && f < s->nf;
        for (int k = 0; k < 3 && ok; k++) {
          vi[k] = s->vidx[3 * f + k];
          ni[k] = s->nidx[3 * f + k];
          mat4_apply(vw->mvp, s->pos + 4 * (size_t)vi[k], clip[k]);
          const double W = clip[k][3];
          ok = ok && W < 0.0;
          const double nx = clip[k][0] / W, ny = clip[k][1] / W, nz = clip[k][2] / W;
          sx[k] = vw->screen[0] * nx + vw->screen[1] * ny + vw->screen[2] * nz + vw->screen[3];
          sy[k] = vw->screen[4] * nx + vw->screen[5] * ny + vw->screen[6] * nz + vw->screen[7];
        }
        if (ok) {
          const double ax = sx[0] - px, ay = sy[0] - py, bx = sx[1] - px, by = sy[1] - py;
          const double cx = sx[2] - px, cy = sy[2] - py;
          e[0] = bx * cy - cx * by;
          e[1] = cx * ay - ax * cy;
          e[2] = ax * by - bx * ay;
          for (int k = 0; k < 3; k++) r[k] = e[k] / clip[k][3];
          R = r[0] + r[1] + r[2];
          ok = R != 0.0 && isfinite(R);
        }
        if (ok) {
          shaded = 1;
          double ms = 0.0;
          for (int k = 0; k < 3; k++) {
            b[k] = r[k] / R;
            l[k] = b[k] > 0.0 ? b[k] : 0.0;
            ms += l[k];
          }
          for (int k = 0; k < 3; k++) l[k] /= ms;
          msum = ms;
          if (texel_in) {
            texel = texel_in[gp];
          } else if (s->tex && s->uv) {
            const double* uv = s->uv + 6 * (size_t)f;
            const double u = l[0] * uv[0] + l[1] * uv[2] + l[2] * uv[4];
            const double vv = l[0] * uv[1] + l[1] * uv[3] + l[2] * uv[5];
            texel = (uint32_t)(wrap_index(vv, s->th) * s->tw + wrap_index(u, s->tw));
          }
          if (texel != NO_FACE && s->tex)
            for (int ch = 0; ch < 4; ch++) t[ch] = s->tex[4 * (size_t)texel + ch];
          for (int k = 0; k < 3; k++) {
            double n4[4];
            mat4_apply(s->world, s->vnrm + 4 * (size_t)ni[k], n4);
            const double len = sqrt(n4[0] * n4[0] + n4[1] * n4[1] + n4[2] * n4[2] + n4[3] * n4[3]);
            for (int j = 0; j < 3; j++) nh[k][j] = n4[j] / len;
            Ik[k] = 0.5 + 0.5 * (nh[k][0] * s->light[0] + nh[k][1] * s->light[1] + nh[k][2] * s->light[2]);
            I += l[k] * Ik[k];
            for (int ch = 0; ch < 3; ch++) col[ch] += l[k] * s->vcol[3 * (size_t)vi[k] + ch];
          }
          for (int ch = 0; ch < 3; ch++) out[ch] = I * col[ch] * t[ch];
          out[3] = t[3];
        }
      }
      if (texel_out) texel_out[gp] = shaded ? texel : NO_FACE;
      double go[4];
      for (int ch = 0; ch < 4; ch++) {
        const double d = out[ch] - (double)tg[ch];
        loss += d * d;
        go[ch] = 2.0 * d;
        if (image) image[4 * gp + ch] = out[ch];
      }
      if (!shaded) continue;
      /* texels */
      if (g_tex && s->tex && texel != NO_FACE) {
        for (int ch = 0; ch < 3; ch++) g_tex[4 * (size_t)texel + ch] += go[ch] * I * col[ch];
        g_tex[4 * (size_t)texel + 3] += go[3];
      }
      double dI = 0.0;
      for (int ch = 0; ch < 3; ch++) dI += go[ch] * col[ch] * t[ch];
      if (g_vcol)
        for (int k = 0; k < 3; k++)
          for (int ch = 0; ch < 3; ch++) g_vcol[3 * (size_t)vi[k] + ch] += go[ch] * I * t[ch] * l[k];
      if (g_light)
        for (int k = 0; k < 3; k++)
          for (int j = 0; j < 3; j++) g_light[j] += dI * 0.5 * l[k] * nh[k][j];
      if (!g_pos) continue;
      /* positions through the barycentrics */
      double G[3];
      for (int k = 0; k < 3; k++) {
        G[k] = dI * Ik[k];
        for (int ch = 0; ch < 3; ch++) G[k] += go[ch] * I * t[ch] * s->vcol[3 * (size_t)vi[k] + ch];
      }
      const double Gl = G[0] * l[0] + G[1] * l[1] + G[2] * l[2];
      double Gb[3];
      for (int k = 0; k < 3; k++) Gb[k] = b[k] > 0.0 ? (G[k] - Gl) / msum : 0.0;
      const double Gbb = Gb[0] * b[0] + Gb[1] * b[1] + Gb[2] * b[2];
      double dE[3], dW[3];
      for (int k = 0; k < 3; k++) {
        const double dr = (Gb[k] - Gbb) / R;
        dE[k] = dr / clip[k][3];
        dW[k] = -dr * r[k] / clip[k][3];
      }
      const double ax = sx[0] - px, ay = sy[0] - py, bx = sx[1] - px, by = sy[1] - py;
      const double cx = sx[2] - px, cy = sy[2] - py;
      const double gx[3] = {-dE[1] * cy + dE[2] * by, dE[0] * cy - dE[2] * ay, -dE[0] * by + dE[1] * ay};
      const double gy[3] = {dE[1] * cx - dE[2] * bx, -dE[0] * cx + dE[2] * ax, dE[0] * bx - dE[1] * ax};
      for (int k = 0; k < 3; k++) {
        const double* c = clip[k];
        const double W = c[3];
        const double gX = (gx[k] * vw->screen[0] + gy[k] * vw->screen[4]) / W;
        const double gY = (gx[k] * vw->screen[1] + gy[k] * vw->screen[5]) / W;
        const double gZ = (gx[k] * vw->screen[2] + gy[k] * vw->screen[6]) / W;
        const double gW = dW[k] - (gX * c[0] + gY * c[1] + gZ * c[2]) / W;
        for (int j = 0; j < 3; j++)
          g_pos[4 * (size_t)vi[k] + j] += gX * vw->mvp[j] + gY * vw->mvp[4 + j] + gZ * vw->mvp[8 + j] +
                                          gW * vw->mvp[12 + j];
      }
    }
    base += npx;
  }
  return loss;
}
