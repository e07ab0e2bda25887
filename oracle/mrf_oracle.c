/*
 * mrf_oracle.c -- CPU restatement of MRFMap's BP and likelihood.
 * TEST INFRASTRUCTURE ONLY (parity checker and timed CPU baseline); the
 * product library never links it.  Parity against the reference itself is
 * UNPINNED (the reference cannot be built here and ships no golden data).
 *
 * Reference anchors (paths inside the MRFMap project):
 *   image clean-up / back-projection   src/GVDBImage.cpp:13-60
 *   camera frame, voxel-unit pose       src/GVDBCamera.cpp:7-32,70-100
 *   brick activation (radius 1)         src/GVDBMRFMap.cpp:117-135
 *   sensor polynomials, potential       src/cuda/gvdbkernels.cu:46-72
 *   cumulative length pass              src/cuda/gvdbkernels.cu:519-571
 *   Pre pass (tau accumulation)         src/cuda/gvdbkernels.cu:689-819
 *   infinity term                       src/cuda/gvdbkernels.cu:1194-1208
 *   Post pass (ray->voxel messages)     src/cuda/gvdbkernels.cu:824-1038
 *   voxel update (FULL_INFERENCE)       src/cuda/gvdbkernels.cu:457-479
 *   schedule                            src/GVDBInference.cpp:100-178
 *   likelihood                          src/cuda/gvdbkernels.cu:183-293,1246-1274
 *
 * GVDB's rayCast/DDA is third-party (gvdb-voxels, fork icoderaven,
 * branch feature/upstream_refactor_merge, unpinned) and absent; voxel
 * traversal here is the published Amanatides & Woo (1987) 3D-DDA.
 *
 * Build with -ffp-contract=off: geometry is specified as separately rounded
 * fp32 operations so the GPU traversal can match it bit for bit.
 */
#include "mrf_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define BRICK 8
#define BVOX 512
/* constants of include/mrfmap/GVDBCommon.cuh:3-8, taken as the fp32 values */
#define F_EPS_F 1e-4f
#define LIKE_EPS_F 1e-3f
#define Z_MIN_F 0.1f
#define Z_MAX_F 10.0f
#define LOOKUP_PX 20
/* __expf flushes below 2^-126, i.e. when 0.5*x^2 > ~87.3: the reference's
 * fp32 potential is exactly zero there.  The restatement makes that cut
 * explicit (and identical on CPU and GPU). */
#define MU_CUTOFF_F 87.0f
#define CUMLEN_GATE_F 0.1f

/* a pinhole camera of one view (the map's own camera comes from params) */
typedef struct {
  int rows, cols;
  float fx, fy, cx, cy;
  /* voxel box of the traversal and activation ([0, 8 NB) unless the view is
   * confined to a scene box) and the endpoint-activation gate */
  int blo[3], bhi[3];
  float glo[3], ghi[3];
} orc_cam;

typedef struct {
  float pose[16];
  float* depth;
  int policy;
  int built_version;
  int retired; /* out of the iterated window (orc_retire_view) */
  /* incidence lists (pixel-major, then along the ray) */
  int nrays;
  int* ray_pix;
  int64_t* ray_off;
  int* meta; /* 5 per ray: n_pre, n_post, r0, rinf, inf_gate */
  int64_t ninc, cap_inc;
  int* vox;
  float* len;
  float* s;
  unsigned char* run;
  double* mu;
  orc_cam cam; /* the view's camera */
  /* per-voxel state over the pool */
  double* m;
  float* cum_len;
  int64_t nvox_alloc;
  int64_t ntouch;
  int* touch;
} orc_view;

struct orc_map {
  orc_params p;
  orc_cam cam; /* the map's camera (params) */
  float* sigma_lut;
  float* bias_lut;
  int G[3], NB[3];
  float hi[3], off[3], inv_res;
  int* brick_slot;
  int nbricks, cap_bricks;
  int* brick_coord;
  double* L;
  double* belief;
  int version;
  orc_view* views;
  int nviews, cap_views;
  int64_t last_updates;
  /* scratch (pool sized) */
  double* q;
  double* lq;
  double* acc;
  int64_t scratch_vox;
  double* pbuf; /* messages of one camera update (orc_update_camera) */
  int64_t pbuf_cap;
  /* the scene box of the view being added (orc_add_view_box) */
  int next_box, box_lo[3], box_hi[3];
};

static int g_threads = 1;
void orc_set_threads(int n) { g_threads = n > 0 ? n : 1; }

static void* xrealloc(void* p, size_t n) {
  void* q = realloc(p, n ? n : 1);
  if (!q) abort();
  return q;
}

/* ---- sensor model (src/cuda/gvdbkernels.cu:46-55) ---------------------- */
static const float* lut_at(const orc_map* m, const orc_cam* cam, const float* lut, int x, int y) {
  /* tile row indexed by the GL row (image flipped on upload,
   * src/GVDBImage.cpp:33 and gvdbkernels.cu:47); a camera of another
   * resolution than the tables' maps its pixel into the tables' grid */
  int ygl = cam->rows - 1 - y;
  int xs = (int)(((int64_t)x * m->p.cols) / cam->cols);
  int ys = (int)(((int64_t)ygl * m->p.rows) / cam->rows);
  int tu = xs / LOOKUP_PX, tv = ys / LOOKUP_PX;
  return lut + ((size_t)tv * m->p.n_tiles_u + tu) * m->p.lookup_n;
}
static float poly_f(const float* c, int n, float z) {
  if (n == 3) {
    float a = (z * z) * c[2];
    float b = z * c[1];
    return (a + b) + c[0];
  }
  return z * c[1] + c[0];
}
static double poly_d(const float* c, int n, double z) {
  if (n == 3) return z * z * (double)c[2] + z * (double)c[1] + (double)c[0];
  return z * (double)c[1] + (double)c[0];
}
/* depth_potential (gvdbkernels.cu:57-72) in FP64: sigma' = 3 sigma(s) */
static double potential_d(const float* sg, const float* bs, int n, double s, double d) {
  double sig3 = 3.0 * poly_d(sg, n, s);
  double diff = fabs(d - (s + poly_d(bs, n, s)));
  double x = diff / sig3;
  return 0.398942 / sig3 * exp(-0.5 * x * x);
}
/* fp32 test shared with the GPU: is the fp32 potential exactly zero? */
static int potential_is_zero_f(const float* sg, const float* bs, int n, float s, float d) {
  float sig3 = 3.0f * poly_f(sg, n, s);
  float diff = fabsf(d - (s + poly_f(bs, n, s)));
  float x = diff / sig3;
  float h = 0.5f * (x * x);
  return !(h <= MU_CUTOFF_F);
}

/* ---- map ----------------------------------------------------------------- */
orc_map* orc_create(const orc_params* p) {
  orc_map* m = (orc_map*)calloc(1, sizeof(orc_map));
  m->p = *p;
  size_t nl = (size_t)p->n_tiles_u * p->n_tiles_v * p->lookup_n;
  m->sigma_lut = (float*)malloc(nl * sizeof(float));
  m->bias_lut = (float*)malloc(nl * sizeof(float));
  memcpy(m->sigma_lut, p->sigma_lut, nl * sizeof(float));
  memcpy(m->bias_lut, p->bias_lut, nl * sizeof(float));
  m->p.sigma_lut = m->sigma_lut;
  m->p.bias_lut = m->bias_lut;
  m->cam.rows = p->rows;
  m->cam.cols = p->cols;
  m->cam.fx = p->fx;
  m->cam.fy = p->fy;
  m->cam.cx = p->cx;
  m->cam.cy = p->cy;
  m->inv_res = 1.0f / p->res;
  for (int a = 0; a < 3; ++a) {
    float g = p->dims[a] / p->res;
    m->hi[a] = g;
    m->G[a] = (int)ceilf(g);
    m->NB[a] = (m->G[a] + 1 + BRICK - 1) / BRICK;
    m->cam.blo[a] = 0;
    m->cam.bhi[a] = BRICK * m->NB[a];
    m->cam.glo[a] = 0.0f;
    m->cam.ghi[a] = g;
  }
  /* src/GVDBCamera.cpp:15-18 / 76-79: x,y centred, z not shifted */
  m->off[0] = (p->dims[0] * 0.5f) / p->res;
  m->off[1] = (p->dims[1] * 0.5f) / p->res;
  m->off[2] = 0.0f;
  size_t nb = (size_t)m->NB[0] * m->NB[1] * m->NB[2];
  m->brick_slot = (int*)malloc(nb * sizeof(int));
  for (size_t i = 0; i < nb; ++i) m->brick_slot[i] = -1;
  return m;
}

static void view_free(orc_view* v) {
  free(v->depth); free(v->ray_pix); free(v->ray_off); free(v->meta);
  free(v->vox); free(v->len); free(v->s); free(v->run); free(v->mu);
  free(v->m); free(v->cum_len); free(v->touch);
}

void orc_destroy(orc_map* m) {
  if (!m) return;
  for (int i = 0; i < m->nviews; ++i) view_free(&m->views[i]);
  free(m->views); free(m->sigma_lut); free(m->bias_lut); free(m->brick_slot);
  free(m->brick_coord); free(m->L); free(m->belief);
  free(m->q); free(m->lq); free(m->acc); free(m->pbuf);
  free(m);
}

int orc_num_views(const orc_map* m) { return m->nviews; }
int orc_num_bricks(const orc_map* m) { return m->nbricks; }
void orc_brick_coords(const orc_map* m, int* out) {
  memcpy(out, m->brick_coord, (size_t)m->nbricks * 3 * sizeof(int));
}
int orc_brick_dims(const orc_map* m, int* out3) {
  for (int a = 0; a < 3; ++a) out3[a] = m->NB[a];
  return m->NB[0] * m->NB[1] * m->NB[2];
}

static int64_t blin(const orc_map* m, int bx, int by, int bz) {
  return ((int64_t)bx * m->NB[1] + by) * m->NB[2] + bz;
}

/* grow per-voxel arrays after new bricks were appended */
static void grow_pool(orc_map* m, int new_nbricks) {
  int64_t nv_old = (int64_t)m->nbricks * BVOX, nv = (int64_t)new_nbricks * BVOX;
  m->L = (double*)xrealloc(m->L, nv * sizeof(double));
  m->belief = (double*)xrealloc(m->belief, nv * sizeof(double));
  double lp = log((double)m->p.prior) - log(1.0 - (double)m->p.prior);
  for (int64_t i = nv_old; i < nv; ++i) { m->L[i] = lp; m->belief[i] = 0.0; }
  for (int c = 0; c < m->nviews; ++c) {
    orc_view* v = &m->views[c];
    v->m = (double*)xrealloc(v->m, nv * sizeof(double));
    v->cum_len = (float*)xrealloc(v->cum_len, nv * sizeof(float));
    for (int64_t i = v->nvox_alloc; i < nv; ++i) { v->m[i] = 0.0; v->cum_len[i] = 0.0f; }
    v->nvox_alloc = nv;
  }
  m->q = (double*)xrealloc(m->q, nv * sizeof(double));
  m->lq = (double*)xrealloc(m->lq, nv * sizeof(double));
  m->acc = (double*)xrealloc(m->acc, nv * sizeof(double));
  m->scratch_vox = nv;
  m->nbricks = new_nbricks;
  m->version++;
}

/* ---- ray set-up (src/GVDBCamera.cpp:7-32; gvdbkernels.cu:1178-1179) ------ */
static void ray_setup(const orc_map* m, const orc_cam* cam, const float* pose, int x, int y, float o[3],
                      float d[3], float* mult) {
  float W = (float)cam->cols, H = (float)cam->rows;
  float ndcx = 2.0f * (((float)x + 0.5f) / W) - 1.0f;
  float ndcy = 2.0f * (((float)y + 0.5f) / H) - 1.0f;
  float rx = ndcx * (cam->cx / cam->fx);
  float ry = ndcy * (cam->cy / cam->fy);
  float dw[3];
  for (int a = 0; a < 3; ++a) {
    float u = pose[a * 4 + 0] * rx;
    float w = pose[a * 4 + 1] * ry;
    dw[a] = (u + w) + pose[a * 4 + 2];
  }
  float n2 = (dw[0] * dw[0] + dw[1] * dw[1]) + dw[2] * dw[2];
  float n = sqrtf(n2);
  for (int a = 0; a < 3; ++a) {
    d[a] = dw[a] / n;
    o[a] = pose[a * 4 + 3] / m->p.res + m->off[a];
  }
  float c0 = pose[2] * d[0];
  float c1 = pose[6] * d[1];
  float c2 = pose[10] * d[2];
  *mult = m->p.res * fabsf((c0 + c1) + c2);
}

/* ---- Amanatides-Woo voxel DDA over the brick-grid box ------------------- */
typedef struct {
  float o[3], d[3], inv[3], tmax[3], tprev;
  int v[3], step[3], lo[3], hi[3];
  int alive, guard;
} dda_t;

/* over the camera's voxel box [blo, bhi) */
static int dda_init(dda_t* r, const orc_cam* cam, const float o[3], const float d[3]) {
  float t0 = 0.0f, t1 = INFINITY;
  for (int a = 0; a < 3; ++a) {
    r->o[a] = o[a]; r->d[a] = d[a];
    r->lo[a] = cam->blo[a];
    r->hi[a] = cam->bhi[a];
    float lo = (float)r->lo[a], E = (float)r->hi[a];
    float tn, tf;
    if (d[a] > 0.0f || d[a] < 0.0f) {
      r->inv[a] = 1.0f / d[a];
      float tA = (lo - o[a]) * r->inv[a];
      float tB = (E - o[a]) * r->inv[a];
      tn = fminf(tA, tB);
      tf = fmaxf(tA, tB);
    } else {
      r->inv[a] = 0.0f;
      if (o[a] < lo || o[a] >= E) return 0;
      tn = -INFINITY;
      tf = INFINITY;
    }
    t0 = fmaxf(t0, tn);
    t1 = fminf(t1, tf);
  }
  if (!(t0 < t1)) return 0;
  for (int a = 0; a < 3; ++a) {
    float pa = o[a] + t0 * d[a];
    int vi = (int)floorf(pa);
    if (vi < r->lo[a]) vi = r->lo[a];
    if (vi > r->hi[a] - 1) vi = r->hi[a] - 1;
    r->v[a] = vi;
    r->step[a] = d[a] > 0.0f ? 1 : (d[a] < 0.0f ? -1 : 0);
    if (r->step[a] > 0)
      r->tmax[a] = ((float)(vi + 1) - o[a]) * r->inv[a];
    else if (r->step[a] < 0)
      r->tmax[a] = ((float)vi - o[a]) * r->inv[a];
    else
      r->tmax[a] = INFINITY;
  }
  r->tprev = t0;
  r->alive = 1;
  r->guard = 2 * ((r->hi[0] - r->lo[0]) + (r->hi[1] - r->lo[1]) + (r->hi[2] - r->lo[2])) + 8;
  return 1;
}

/* emits the current voxel, its segment length and exit parameter, then steps */
static int dda_next(dda_t* r, int vout[3], float* len, float* tin, float* texit) {
  if (!r->alive || r->guard-- <= 0) return 0;
  int a = (r->tmax[0] <= r->tmax[1] && r->tmax[0] <= r->tmax[2]) ? 0
          : (r->tmax[1] <= r->tmax[2] ? 1 : 2);
  float te = r->tmax[a];
  float l = te - r->tprev;
  if (l < 0.0f) l = 0.0f;
  vout[0] = r->v[0]; vout[1] = r->v[1]; vout[2] = r->v[2];
  *len = l;
  *tin = r->tprev;
  *texit = te;
  r->tprev = fmaxf(r->tprev, te);
  r->v[a] += r->step[a];
  if (r->v[a] < r->lo[a] || r->v[a] >= r->hi[a]) {
    r->alive = 0;
  } else {
    float nb = r->step[a] > 0 ? (float)(r->v[a] + 1) : (float)r->v[a];
    r->tmax[a] = (nb - r->o[a]) * r->inv[a];
  }
  return 1;
}

static int vox_id(const orc_map* m, const int v[3], int64_t* lin_out) {
  int bx = v[0] >> 3, by = v[1] >> 3, bz = v[2] >> 3;
  int64_t lin = blin(m, bx, by, bz);
  *lin_out = lin;
  int slot = m->brick_slot[lin];
  if (slot < 0) return -1;
  int lx = v[0] & 7, ly = v[1] & 7, lz = v[2] & 7;
  return slot * BVOX + ((lx * BRICK + ly) * BRICK + lz);
}

/* ---- image clean-up (src/GVDBImage.cpp:32-40) ---------------------------- */
static void clean_depth(const orc_cam* cam, const float* in, float* out) {
  int H = cam->rows, W = cam->cols;
  for (int i = 0; i < H * W; ++i) out[i] = isfinite(in[i]) ? in[i] : -1.0f;
  if (H == 480 && W == 848) {
    for (int y = 0; y < H; ++y)
      for (int x = 0; x < W; ++x)
        if (x < 24 || x >= W - 24 || y < 20 || y >= H - 20) out[y * W + x] = -1.0f;
  }
}

/* ---- activation (src/GVDBCamera.cpp:70-100; src/GVDBMRFMap.cpp:117-135) -- */
static int floordiv8(int v) { return v >= 0 ? v / 8 : -((-v + 7) / 8); }

static void mark_point_bricks(const orc_map* m, const orc_cam* cam, const float pv[3], unsigned char* flag) {
  int lo[3], hi[3];
  for (int a = 0; a < 3; ++a) {
    int vi = (int)floorf(pv[a]);
    lo[a] = floordiv8(vi - 1);
    hi[a] = floordiv8(vi + 1);
    if (lo[a] < cam->blo[a] / BRICK) lo[a] = cam->blo[a] / BRICK;
    if (hi[a] > cam->bhi[a] / BRICK - 1) hi[a] = cam->bhi[a] / BRICK - 1;
  }
  for (int bx = lo[0]; bx <= hi[0]; ++bx)
    for (int by = lo[1]; by <= hi[1]; ++by)
      for (int bz = lo[2]; bz <= hi[2]; ++bz) flag[blin(m, bx, by, bz)] = 1;
}

static void activate_view(orc_map* m, const orc_cam* cam, const float* pose, const float* depth,
                          int policy) {
  int H = cam->rows, W = cam->cols;
  size_t nb = (size_t)m->NB[0] * m->NB[1] * m->NB[2];
  unsigned char* flag = (unsigned char*)calloc(nb, 1);
  for (int y = 0; y < H; ++y) {
    for (int x = 0; x < W; ++x) {
      float d = depth[y * W + x];
      if (!(d > 0.0f)) continue;
      /* back-projection uses fx for both axes and integer pixel coords
       * (src/GVDBImage.cpp:48-56) */
      float f = d / cam->fx;
      float X = f * ((float)x - cam->cx);
      float Y = f * ((float)y - cam->cy);
      float Z = d;
      float pv[3];
      int inside = 1;
      for (int a = 0; a < 3; ++a) {
        float u = pose[a * 4 + 0] * X;
        float w = pose[a * 4 + 1] * Y;
        float z = pose[a * 4 + 2] * Z;
        float pw = ((u + w) + z) + pose[a * 4 + 3];
        pv[a] = pw * m->inv_res + m->off[a];
        if (!(pv[a] >= cam->glo[a] && pv[a] < cam->ghi[a])) inside = 0;
      }
      if (inside) mark_point_bricks(m, cam, pv, flag);
      if (policy == ORC_ACT_FULL_RAY) {
        /* every brick the ray crosses up to the brick run where the Pre
         * pass stops: at the exit s of a run's last voxel,
         * s + bias(s) > d + 3 sigma(s) (the stop test of build_ray) */
        float o[3], dr[3], mult;
        ray_setup(m, cam, pose, x, y, o, dr, &mult);
        const float* sg = lut_at(m, cam, m->sigma_lut, x, y);
        const float* bs = lut_at(m, cam, m->bias_lut, x, y);
        const int n = m->p.lookup_n;
        dda_t r;
        if (dda_init(&r, cam, o, dr)) {
          int v[3];
          float l, tin, te, s_last = 0.0f;
          int64_t cur = -1;
          while (dda_next(&r, v, &l, &tin, &te)) {
            int64_t lin = blin(m, v[0] >> 3, v[1] >> 3, v[2] >> 3);
            if (lin != cur) {
              if (cur >= 0) {
                float lhs = s_last + poly_f(bs, n, s_last);
                float rhs = d + 3.0f * poly_f(sg, n, s_last);
                if (lhs > rhs) break;
              }
              flag[lin] = 1;
              cur = lin;
            }
            s_last = te * mult;
          }
        }
      }
    }
  }
  /* new bricks take slots in increasing linear brick index */
  int add = 0;
  for (size_t i = 0; i < nb; ++i)
    if (flag[i] && m->brick_slot[i] < 0) ++add;
  if (add) {
    int n0 = m->nbricks;
    m->brick_coord = (int*)xrealloc(m->brick_coord, (size_t)(n0 + add) * 3 * sizeof(int));
    int s = n0;
    for (size_t i = 0; i < nb; ++i) {
      if (flag[i] && m->brick_slot[i] < 0) {
        m->brick_slot[i] = s;
        int bz = (int)(i % m->NB[2]);
        int by = (int)((i / m->NB[2]) % m->NB[1]);
        int bx = (int)(i / ((size_t)m->NB[2] * m->NB[1]));
        m->brick_coord[s * 3 + 0] = bx;
        m->brick_coord[s * 3 + 1] = by;
        m->brick_coord[s * 3 + 2] = bz;
        ++s;
      }
    }
    grow_pool(m, n0 + add);
  }
  free(flag);
}

int orc_add_view_camera(orc_map* m, const float* pose, const float* depth, int policy, int rows, int cols,
                        float fx, float fy, float cx, float cy) {
  if (m->nviews == m->cap_views) {
    m->cap_views = m->cap_views ? 2 * m->cap_views : 8;
    m->views = (orc_view*)xrealloc(m->views, (size_t)m->cap_views * sizeof(orc_view));
  }
  orc_view* v = &m->views[m->nviews];
  memset(v, 0, sizeof(*v));
  memcpy(v->pose, pose, sizeof(v->pose));
  v->cam.rows = rows;
  v->cam.cols = cols;
  v->cam.fx = fx;
  v->cam.fy = fy;
  v->cam.cx = cx;
  v->cam.cy = cy;
  for (int a = 0; a < 3; ++a) {
    v->cam.blo[a] = m->cam.blo[a];
    v->cam.bhi[a] = m->cam.bhi[a];
    v->cam.glo[a] = m->cam.glo[a];
    v->cam.ghi[a] = m->cam.ghi[a];
  }
  if (m->next_box) {
    /* a view confined to a scene box (orc_add_view_box) */
    for (int a = 0; a < 3; ++a) {
      v->cam.blo[a] = BRICK * m->box_lo[a];
      v->cam.bhi[a] = BRICK * m->box_hi[a];
      v->cam.glo[a] = (float)v->cam.blo[a];
      v->cam.ghi[a] = fminf(m->hi[a], (float)v->cam.bhi[a]);
    }
    m->next_box = 0;
  }
  v->depth = (float*)malloc((size_t)rows * cols * sizeof(float));
  clean_depth(&v->cam, depth, v->depth);
  v->policy = policy;
  v->built_version = -1;
  int64_t nv = (int64_t)m->nbricks * BVOX;
  v->m = (double*)calloc((size_t)(nv ? nv : 1), sizeof(double));
  v->cum_len = (float*)calloc((size_t)(nv ? nv : 1), sizeof(float));
  v->nvox_alloc = nv;
  m->nviews++;
  activate_view(m, &v->cam, v->pose, v->depth, policy);
  return m->nviews - 1;
}

int orc_add_view_box(orc_map* m, const float* pose, const float* depth, int policy, int rows, int cols, float fx,
                     float fy, float cx, float cy, const int brick_lo[3], const int brick_hi[3]) {
  for (int a = 0; a < 3; ++a) {
    if (brick_lo[a] < 0 || brick_hi[a] > m->NB[a] || brick_lo[a] >= brick_hi[a]) return -1;
    m->box_lo[a] = brick_lo[a];
    m->box_hi[a] = brick_hi[a];
  }
  m->next_box = 1;
  return orc_add_view_camera(m, pose, depth, policy, rows, cols, fx, fy, cx, cy);
}

int orc_add_view(orc_map* m, const float* pose, const float* depth, int policy) {
  return orc_add_view_camera(m, pose, depth, policy, m->cam.rows, m->cam.cols, m->cam.fx, m->cam.fy,
                             m->cam.cx, m->cam.cy);
}

int orc_view_pixels(const orc_map* m, int view) {
  if (view < 0 || view >= m->nviews) return 0;
  return m->views[view].cam.rows * m->views[view].cam.cols;
}

static double belief_of(double L);

/* Moving a camera first removes its messages from the total log-odds (the
 * reference subtracts the camera's ray contributions before re-activating,
 * src/GVDBInference.cpp:66-82). */
int orc_set_pose(orc_map* m, int view, const float* pose, int policy) {
  if (view < 0 || view >= m->nviews) return -1;
  orc_view* v = &m->views[view];
  for (int64_t i = 0; i < v->nvox_alloc; ++i) {
    if (v->m[i] != 0.0) {
      m->L[i] -= v->m[i];
      m->belief[i] = belief_of(m->L[i]);
      v->m[i] = 0.0;
    }
  }
  memcpy(m->views[view].pose, pose, 16 * sizeof(float));
  m->views[view].built_version = -1;
  activate_view(m, &m->views[view].cam, m->views[view].pose, m->views[view].depth, policy);
  return 0;
}

/* ---- per-view incidence lists ------------------------------------------- */
static void push_inc(orc_view* v, int vox, float len, float s, unsigned char run) {
  if (v->ninc == v->cap_inc) {
    v->cap_inc = v->cap_inc ? 2 * v->cap_inc : 4096;
    v->vox = (int*)xrealloc(v->vox, (size_t)v->cap_inc * sizeof(int));
    v->len = (float*)xrealloc(v->len, (size_t)v->cap_inc * sizeof(float));
    v->s = (float*)xrealloc(v->s, (size_t)v->cap_inc * sizeof(float));
    v->run = (unsigned char*)xrealloc(v->run, (size_t)v->cap_inc);
  }
  v->vox[v->ninc] = vox;
  v->len[v->ninc] = len;
  v->s[v->ninc] = s;
  v->run[v->ninc] = run;
  v->ninc++;
}

/* One pixel's BP incidence list: active voxels in ray order, grouped in brick
 * runs; after each run the stop rules of gvdbkernels.cu:816 (Pre, '>') and
 * :1035 / :568 (Post and cumulative length, '>=') are evaluated at the exit
 * depth of the run's last voxel. */
static void build_ray(orc_map* m, orc_view* v, int x, int y, float d, int* meta) {
  const float* sg = lut_at(m, &v->cam, m->sigma_lut, x, y);
  const float* bs = lut_at(m, &v->cam, m->bias_lut, x, y);
  int n = m->p.lookup_n;
  float o[3], dr[3], mult;
  ray_setup(m, &v->cam, v->pose, x, y, o, dr, &mult);
  int64_t start = v->ninc;
  int count = 0, n_post = -1, n_pre = -1;
  int run_open = 0;
  int64_t cur_lin = -1;
  float s_last = 0.0f;
  dda_t r;
  if (dda_init(&r, &v->cam, o, dr)) {
    int vv[3];
    float l, tin, te;
    while (dda_next(&r, vv, &l, &tin, &te)) {
      int64_t lin;
      int id = vox_id(m, vv, &lin);
      if (lin != cur_lin) {
        if (run_open) {
          run_open = 0;
          float lhs = s_last + poly_f(bs, n, s_last);
          float rhs = d + 3.0f * poly_f(sg, n, s_last);
          if (n_post < 0 && lhs >= rhs) n_post = count;
          if (lhs > rhs) { n_pre = count; break; }
        }
        cur_lin = lin;
      }
      if (id < 0) continue;
      float s = te * mult;
      push_inc(v, id, l, s, (unsigned char)(run_open ? 0 : 1));
      run_open = 1;
      s_last = s;
      ++count;
    }
    if (n_pre < 0 && run_open) {
      float lhs = s_last + poly_f(bs, n, s_last);
      float rhs = d + 3.0f * poly_f(sg, n, s_last);
      if (n_post < 0 && lhs >= rhs) n_post = count;
      if (lhs > rhs) n_pre = count;
    }
  }
  int gate = 0;
  if (n_pre < 0) {
    n_pre = count;
    /* infinity term (gvdbkernels.cu:1196-1208): only when Pre never stopped */
    if (count > 0) gate = d > s_last + poly_f(bs, n, s_last);
  }
  if (n_post < 0) n_post = count;
  /* drop incidences past the Pre stop (none are pushed after the break) */
  v->ninc = start + n_pre;
  /* Pre-pass carries its visibility across bricks only once the
   * accumulated tau is non-zero (gvdbkernels.cu:708-715): the effective
   * start is the first run holding a voxel with a non-zero potential. */
  int r0 = n_pre, rinf = 0, last_run = 0;
  for (int i = 0; i < n_pre; ++i) {
    if (v->run[start + i]) last_run = i;
    if (r0 == n_pre && !potential_is_zero_f(sg, bs, n, v->s[start + i], d)) {
      int k = i;
      while (k > 0 && !v->run[start + k]) --k;
      r0 = k;
    }
  }
  rinf = (r0 < n_pre) ? r0 : last_run;
  meta[0] = n_pre;
  meta[1] = n_post;
  meta[2] = r0;
  meta[3] = rinf;
  meta[4] = gate;
}

static void build_view(orc_map* m, int c) {
  orc_view* v = &m->views[c];
  int H = v->cam.rows, W = v->cam.cols;
  free(v->ray_pix); free(v->ray_off); free(v->meta); free(v->mu); free(v->touch);
  v->ray_pix = (int*)malloc((size_t)H * W * sizeof(int));
  v->ray_off = (int64_t*)malloc((size_t)H * W * sizeof(int64_t));
  v->meta = (int*)malloc((size_t)H * W * 5 * sizeof(int));
  v->nrays = 0;
  v->ninc = 0;
  for (int y = 0; y < H; ++y) {
    for (int x = 0; x < W; ++x) {
      float d = v->depth[y * W + x];
      if (!(d > 0.0f)) continue; /* gvdbkernels.cu:1170-1173 */
      int64_t off = v->ninc;
      int meta[5];
      build_ray(m, v, x, y, d, meta);
      if (meta[0] == 0) continue;
      v->ray_pix[v->nrays] = y * W + x;
      v->ray_off[v->nrays] = off;
      memcpy(&v->meta[v->nrays * 5], meta, sizeof(meta));
      v->nrays++;
    }
  }
  /* potentials (FP64) and cumulative lengths (summed in FP64, rounded once
   * to fp32: the value then does not depend on the order of the additions,
   * which the reference leaves to float atomics) */
  v->mu = (double*)malloc((size_t)(v->ninc ? v->ninc : 1) * sizeof(double));
  int64_t nv = (int64_t)m->nbricks * BVOX;
  double* cum_d = (double*)calloc((size_t)(nv ? nv : 1), sizeof(double));
  unsigned char* seen = (unsigned char*)calloc((size_t)(nv ? nv : 1), 1);
  v->touch = (int*)malloc((size_t)(nv ? nv : 1) * sizeof(int));
  v->ntouch = 0;
  for (int r = 0; r < v->nrays; ++r) {
    int pix = v->ray_pix[r];
    int x = pix % W, y = pix / W;
    const float* sg = lut_at(m, &v->cam, m->sigma_lut, x, y);
    const float* bs = lut_at(m, &v->cam, m->bias_lut, x, y);
    float d = v->depth[pix];
    const int* me = &v->meta[r * 5];
    for (int i = 0; i < me[0]; ++i) {
      int64_t k = v->ray_off[r] + i;
      float s = v->s[k];
      v->mu[k] = potential_is_zero_f(sg, bs, m->p.lookup_n, s, d)
                     ? 0.0
                     : potential_d(sg, bs, m->p.lookup_n, (double)s, (double)d);
      if (i < me[1]) cum_d[v->vox[k]] += (double)v->len[k];
      if (!seen[v->vox[k]]) {
        seen[v->vox[k]] = 1;
        v->touch[v->ntouch++] = v->vox[k];
      }
    }
  }
  free(seen);
  for (int64_t i = 0; i < nv; ++i) v->cum_len[i] = (float)cum_d[i];
  free(cum_d);
  v->built_version = m->version;
}

static void ensure_built(orc_map* m, int c) {
  if (!m->views[c].retired && m->views[c].built_version != m->version) build_view(m, c);
}

int64_t orc_view_num_incidences(orc_map* m, int view) {
  ensure_built(m, view);
  return m->views[view].ninc;
}

int orc_view_trace(orc_map* m, int view, int* ray_pix, int64_t* ray_off, int* ray_meta,
                   int* inc_vox, float* inc_len, float* inc_s, unsigned char* inc_run,
                   double* inc_mu) {
  ensure_built(m, view);
  orc_view* v = &m->views[view];
  if (ray_pix) memcpy(ray_pix, v->ray_pix, (size_t)v->nrays * sizeof(int));
  if (ray_off) memcpy(ray_off, v->ray_off, (size_t)v->nrays * sizeof(int64_t));
  if (ray_meta) memcpy(ray_meta, v->meta, (size_t)v->nrays * 5 * sizeof(int));
  if (inc_vox) memcpy(inc_vox, v->vox, (size_t)v->ninc * sizeof(int));
  if (inc_len) memcpy(inc_len, v->len, (size_t)v->ninc * sizeof(float));
  if (inc_s) memcpy(inc_s, v->s, (size_t)v->ninc * sizeof(float));
  if (inc_run) memcpy(inc_run, v->run, (size_t)v->ninc);
  if (inc_mu) memcpy(inc_mu, v->mu, (size_t)v->ninc * sizeof(double));
  return v->nrays;
}

/* ---- BP ------------------------------------------------------------------ */
static const double F_EPS = (double)F_EPS_F;

static double clampd(double x, double lo, double hi) { return x < lo ? lo : (x > hi ? hi : x); }

/* cavity probabilities q = P(empty) excluding this camera's own message
 * (gvdbkernels.cu:764-773) */
static void prepare_q(orc_map* m, orc_view* v) {
  for (int64_t k = 0; k < v->ntouch; ++k) {
    int vx = v->touch[k];
    double eta = m->L[vx] - v->m[vx];
    double q = clampd(1.0 / (1.0 + exp(eta)), F_EPS, 1.0 - F_EPS);
    m->q[vx] = q;
    m->lq[vx] = log(q);
  }
}

/* Pre + infinity + Post for every ray of a view; writes p_i into pout */
static void ray_messages(orc_map* m, orc_view* v, int fix_reset, double* pout) {
  const double* Q = m->q;
  const double* LQ = m->lq;
#pragma omp parallel for schedule(dynamic, 64) num_threads(g_threads)
  for (int r = 0; r < v->nrays; ++r) {
    const int* me = &v->meta[r * 5];
    int64_t off = v->ray_off[r];
    int n_pre = me[0], n_post = me[1];
    int r0 = fix_reset ? 0 : me[2];
    int rinf = fix_reset ? 0 : me[3];
    const int* vx = v->vox + off;
    const float* ln = v->len + off;
    const double* mu = v->mu + off;
    /* Pre (gvdbkernels.cu:773-796) */
    double A = 0.0, T = 0.0;
    for (int i = r0; i < n_pre; ++i) {
      A += (double)ln[i] * LQ[vx[i]];
      if (mu[i] != 0.0) T += exp(A) * (1.0 - Q[vx[i]]) * mu[i];
    }
    /* infinity term: visibility at the end of Pre (gvdbkernels.cu:1205) */
    if (me[4]) {
      double Ai = 0.0;
      for (int i = rinf; i < n_pre; ++i) Ai += (double)ln[i] * LQ[vx[i]];
      T += exp(Ai);
    }
    /* Post (gvdbkernels.cu:919-943) */
    A = 0.0;
    double F = 0.0;
    for (int i = 0; i < n_post; ++i) {
      double q = Q[vx[i]];
      A += (double)ln[i] * LQ[vx[i]];
      double V = exp(A);
      double tau = V * (1.0 - q) * mu[i];
      double R = T - F - tau;
      double mu1 = F + V * mu[i];
      double mu0 = F + R / q;
      double p = clampd(mu1 / (mu1 + mu0 + 1e-7), F_EPS, 1.0 - F_EPS);
      pout[off + i] = p;
      F += tau;
    }
  }
}

/* factor->voxel aggregation and belief (gvdbkernels.cu:457-479) */
static void accumulate(orc_map* m, orc_view* v, const double* p) {
  for (int64_t k = 0; k < v->ntouch; ++k) m->acc[v->touch[k]] = 0.0;
  for (int r = 0; r < v->nrays; ++r) {
    int64_t off = v->ray_off[r];
    int n_post = v->meta[r * 5 + 1];
    for (int i = 0; i < n_post; ++i) m->acc[v->vox[off + i]] += p[off + i] * (double)v->len[off + i];
  }
}

static double belief_of(double L) {
  return 1.0 - clampd(1.0 / (1.0 + exp(L)), F_EPS, 1.0 - F_EPS);
}

static void update_view(orc_map* m, orc_view* v, double* dL) {
  for (int64_t k = 0; k < v->ntouch; ++k) {
    int vx = v->touch[k];
    if (!(v->cum_len[vx] > CUMLEN_GATE_F)) continue;
    double a = clampd(m->acc[vx] / (double)v->cum_len[vx], F_EPS, 1.0 - F_EPS);
    double mn = log(a) - log(1.0 - a);
    if (dL) {
      dL[vx] += mn - v->m[vx];
    } else {
      m->L[vx] += mn - v->m[vx];
      m->belief[vx] = belief_of(m->L[vx]);
    }
    v->m[vx] = mn;
  }
}

void orc_infer(orc_map* m, const int* ids, int n_ids, int iters, int flags) {
  if (iters <= 0) iters = 1;
  if (!(flags & ORC_INCREMENTAL)) {
    /* src/GVDBInference.cpp:128-133: zero the selected cameras' channels */
    for (int k = 0; k < n_ids; ++k) {
      int c = ids[k];
      if (c < 0 || c >= m->nviews) continue;
      orc_view* v = &m->views[c];
      if (v->retired) continue;
      for (int64_t i = 0; i < v->nvox_alloc; ++i) v->m[i] = 0.0;
    }
  }
  int64_t maxinc = 1;
  for (int c = 0; c < m->nviews; ++c) {
    ensure_built(m, c);
    if (!m->views[c].retired && m->views[c].ninc > maxinc) maxinc = m->views[c].ninc;
  }
  int fix = (flags & ORC_FIX_PRE_RESET) != 0;
  int64_t nv = (int64_t)m->nbricks * BVOX;
  m->last_updates = 0;
  if (!(flags & ORC_JACOBI)) {
    /* Gauss-Seidel over every camera (src/GVDBInference.cpp:155-167) */
    double* p = (double*)malloc((size_t)maxinc * sizeof(double));
    for (int it = 0; it < iters; ++it) {
      for (int c = 0; c < m->nviews; ++c) {
        orc_view* v = &m->views[c];
        if (v->retired) continue;
        prepare_q(m, v);
        ray_messages(m, v, fix, p);
        accumulate(m, v, p);
        update_view(m, v, NULL);
        for (int r = 0; r < v->nrays; ++r) m->last_updates += v->meta[r * 5 + 1];
      }
    }
    free(p);
  } else {
    double* dL = (double*)calloc((size_t)(nv ? nv : 1), sizeof(double));
    unsigned char* hit = (unsigned char*)calloc((size_t)(nv ? nv : 1), 1);
    double** ps = (double**)malloc((size_t)m->nviews * sizeof(double*));
    for (int c = 0; c < m->nviews; ++c)
      ps[c] = (double*)malloc((size_t)(m->views[c].ninc ? m->views[c].ninc : 1) * sizeof(double));
    for (int it = 0; it < iters; ++it) {
      for (int c = 0; c < m->nviews; ++c) {
        if (m->views[c].retired) continue;
        prepare_q(m, &m->views[c]);
        ray_messages(m, &m->views[c], fix, ps[c]);
      }
      for (int c = 0; c < m->nviews; ++c) {
        orc_view* v = &m->views[c];
        if (v->retired) continue;
        accumulate(m, v, ps[c]);
        update_view(m, v, dL);
        for (int64_t k = 0; k < v->ntouch; ++k)
          if (v->cum_len[v->touch[k]] > CUMLEN_GATE_F) hit[v->touch[k]] = 1;
        for (int r = 0; r < v->nrays; ++r) m->last_updates += v->meta[r * 5 + 1];
      }
      for (int64_t i = 0; i < nv; ++i) {
        if (hit[i]) {
          m->L[i] += dL[i];
          m->belief[i] = belief_of(m->L[i]);
          dL[i] = 0.0;
          hit[i] = 0;
        }
      }
    }
    for (int c = 0; c < m->nviews; ++c) free(ps[c]);
    free(ps);
    free(dL);
    free(hit);
  }
}

void orc_retire_view(orc_map* m, int c) {
  if (c < 0 || c >= m->nviews) return;
  /* its messages stay in L (L is only ever moved by message changes); the
   * view is no longer traced or iterated */
  m->views[c].retired = 1;
}

void orc_build_all(orc_map* m) {
  /* views are independent: each build touches its own view only */
#pragma omp parallel for schedule(dynamic, 1) num_threads(g_threads)
  for (int c = 0; c < m->nviews; ++c) ensure_built(m, c);
}

int64_t orc_update_camera(orc_map* m, int c, int flags) {
  if (c < 0 || c >= m->nviews) return -1;
  ensure_built(m, c);
  orc_view* v = &m->views[c];
  if (v->ninc > m->pbuf_cap) {
    free(m->pbuf);
    m->pbuf = (double*)malloc((size_t)v->ninc * sizeof(double));
    m->pbuf_cap = v->ninc;
  }
  /* the body of the Gauss-Seidel camera loop (src/GVDBInference.cpp:155-167) */
  prepare_q(m, v);
  ray_messages(m, v, (flags & ORC_FIX_PRE_RESET) != 0, m->pbuf);
  accumulate(m, v, m->pbuf);
  update_view(m, v, NULL);
  int64_t n = 0;
  for (int r = 0; r < v->nrays; ++r) n += v->meta[r * 5 + 1];
  return n;
}

int64_t orc_last_updates(const orc_map* m) { return m->last_updates; }

void orc_get_beliefs(const orc_map* m, float* out) {
  int64_t nv = (int64_t)m->nbricks * BVOX;
  for (int64_t i = 0; i < nv; ++i) out[i] = (float)m->belief[i];
}
void orc_get_beliefs_f64(const orc_map* m, double* out) {
  memcpy(out, m->belief, (size_t)m->nbricks * BVOX * sizeof(double));
}
void orc_get_logodds_f64(const orc_map* m, double* out) {
  memcpy(out, m->L, (size_t)m->nbricks * BVOX * sizeof(double));
}
void orc_set_beliefs(orc_map* m, const float* in) {
  int64_t nv = (int64_t)m->nbricks * BVOX;
  for (int64_t i = 0; i < nv; ++i) m->belief[i] = (double)in[i];
}

int orc_trace_pixel(const orc_map* m, const float* pose, int x, int y, int* vox, float* len,
                    float* s, int max) {
  float o[3], dr[3], mult;
  ray_setup(m, &m->cam, pose, x, y, o, dr, &mult);
  dda_t r;
  int n = 0;
  if (!dda_init(&r, &m->cam, o, dr)) return 0;
  int vv[3];
  float l, tin, te;
  while (dda_next(&r, vv, &l, &tin, &te)) {
    int64_t lin;
    int id = vox_id(m, vv, &lin);
    if (id < 0) continue;
    if (n < max) {
      if (vox) vox[n] = id;
      if (len) len[n] = l;
      if (s) s[n] = te * mult;
    }
    ++n;
  }
  return n;
}

/* ---- standard log-odds ray insertion ------------------------------------
 * The occupancy update of classic occupancy mapping (as OctoMap's
 * insertPointCloud applies it: every voxel a ray crosses before its
 * endpoint gets the miss log-odds, the voxel holding the endpoint the hit
 * log-odds, each clamped), over the map's active voxels with the same
 * traversal.  Not part of MRFMap: a CPU baseline for the insertion-style
 * mapping the paper compares against (OctoMap itself is absent here).
 * Single-threaded, in pixel order.  Returns the voxel updates made. */
int64_t orc_insert_logodds(const orc_map* m, const float* pose, const float* depth, float l_hit,
                           float l_miss, float l_min, float l_max, double* L) {
  int64_t n = 0;
  for (int y = 0; y < m->cam.rows; ++y)
    for (int x = 0; x < m->cam.cols; ++x) {
      const float d = depth[(int64_t)y * m->cam.cols + x];
      if (!(d > 0.0f)) continue;
      float o[3], dr[3], mult;
      ray_setup(m, &m->cam, pose, x, y, o, dr, &mult);
      dda_t r;
      if (!dda_init(&r, &m->cam, o, dr)) continue;
      int vv[3];
      float l, tin, te;
      while (dda_next(&r, vv, &l, &tin, &te)) {
        int64_t lin;
        const int id = vox_id(m, vv, &lin);
        const int hit = te * mult >= d;
        if (id >= 0) {
          double v = L[id] + (hit ? l_hit : l_miss);
          L[id] = v < l_min ? l_min : (v > l_max ? l_max : v);
          ++n;
        }
        if (hit) break;
      }
    }
  return n;
}

/* ---- likelihood (gvdbkernels.cu:183-293, 1246-1274) ---------------------- */
static double like_pixel(const orc_map* m, const float* pose, int x, int y, float d) {
  const float* sg = lut_at(m, &m->cam, m->sigma_lut, x, y);
  const float* bs = lut_at(m, &m->cam, m->bias_lut, x, y);
  int n = m->p.lookup_n;
  const double LE = (double)LIKE_EPS_F;
  float o[3], dr[3], mult;
  ray_setup(m, &m->cam, pose, x, y, o, dr, &mult);
  double A = 0.0, Vprev = 1.0, sum = 0.0, prev_s = 0.0;
  int first_run = 1, run_open = 0;
  int64_t cur_lin = -1;
  float s_last = 0.0f;
  dda_t r;
  if (dda_init(&r, &m->cam, o, dr)) {
    int vv[3];
    float l, tin, te;
    while (dda_next(&r, vv, &l, &tin, &te)) {
      int64_t lin;
      int id = vox_id(m, vv, &lin);
      if (lin != cur_lin) {
        if (run_open) {
          run_open = 0;
          /* brick exit stores s + bias(s) as the next brick's previous s
           * (gvdbkernels.cu:209,292) */
          prev_s = (double)s_last + poly_d(bs, n, (double)s_last);
        }
        cur_lin = lin;
      }
      if (id < 0) continue;
      if (!run_open) {
        run_open = 1;
        if (first_run) {
          prev_s = (double)(tin * mult);
          first_run = 0;
        }
      }
      double p = m->belief[id];
      double alpha = -log(1.0 - p);
      A += -alpha * (double)l;
      double V = exp(A);
      float sf = te * mult;
      double sd = (double)sf;
      double P;
      if (sf < Z_MIN_F) {
        P = 0.0;
      } else {
        float pd = (sf + poly_f(bs, n, sf)) - d;
        if (fabsf(pd) <= 3.0f * poly_f(sg, n, sf))
          P = (1.0 - LE) * 0.5 *
              (potential_d(sg, bs, n, sd, (double)d) + potential_d(sg, bs, n, prev_s, (double)d));
        else
          P = LE;
      }
      sum += (Vprev - V) * P;
      Vprev = V;
      prev_s = sd;
      s_last = sf;
    }
  }
  sum += Vprev * (d >= Z_MAX_F ? 1.0 - LE : LE);
  return log(sum);
}

double orc_likelihood(const orc_map* m, const float* pose, const float* depth, float* out_img) {
  int H = m->p.rows, W = m->p.cols;
  float* dep = (float*)malloc((size_t)H * W * sizeof(float));
  clean_depth(&m->cam, depth, dep);
  double total = 0.0;
#pragma omp parallel for schedule(dynamic, 16) reduction(+ : total) num_threads(g_threads)
  for (int y = 0; y < H; ++y) {
    for (int x = 0; x < W; ++x) {
      float d = dep[y * W + x];
      double v = 0.0;
      if (d > 0.0f) v = like_pixel(m, pose, x, y, d);
      if (out_img) out_img[y * W + x] = (float)v;
      total += v;
    }
  }
  free(dep);
  return total;
}

/* ---- evaluation renders --------------------------------------------------- */
/* The likelihood traversal (every active brick to the volume exit) with the
 * extra state the reference's evaluation kernels keep in hit/norm/clr. */
static float render_pixel(const orc_map* m, int mode, const float* pose, int x, int y, float d,
                          float thresh) {
  const float* sg = lut_at(m, &m->cam, m->sigma_lut, x, y);
  const float* bs = lut_at(m, &m->cam, m->bias_lut, x, y);
  int n = m->p.lookup_n;
  float o[3], dr[3], mult;
  ray_setup(m, &m->cam, pose, x, y, o, dr, &mult);
  double A = 0.0, Vprev = 1.0, sum = 0.0;
  double peak = 0.0;   /* hit.x: peak of (V_prev - V) / l */
  int peak_ok = 0;     /* hit.y */
  int occ = -1;        /* norm.y (occupancy-threshold kernel) */
  int any = 0;
  float s_last = 0.0f;
  int64_t cur_lin = -1;
  int run_open = 0;
  dda_t r;
  if (dda_init(&r, &m->cam, o, dr)) {
    int vv[3];
    float l, tin, te;
    while (dda_next(&r, vv, &l, &tin, &te)) {
      int64_t lin;
      int id = vox_id(m, vv, &lin);
      if (lin != cur_lin) {
        if (run_open && mode == 2 && s_last >= d) return 0.0f; /* passed the return: miss */
        run_open = 0;
        cur_lin = lin;
      }
      if (id < 0) continue;
      run_open = 1;
      any = 1;
      double p = m->belief[id];
      float sf = te * mult;
      s_last = sf;
      if (mode == 2) {
        if ((float)p >= thresh) return fabsf(sf - d) <= m->p.res ? 1.0f : 2.0f;
        continue;
      }
      double dA = -(-log(1.0 - p)) * (double)l;
      A += dA;
      double V = exp(A);
      if (mode == 0) {
        /* z-depth of the voxel's corner (GVDB atlas-to-world position) */
        double zc = fabs((double)pose[2] * ((double)vv[0] - o[0]) + (double)pose[6] * ((double)vv[1] - o[1]) +
                         (double)pose[10] * ((double)vv[2] - o[2])) * (double)m->p.res;
        sum += (Vprev - V) * zc;
      } else {
        float pd = (sf + poly_f(bs, n, sf)) - d;
        double w = (Vprev - V) / (double)l;
        if (mode == 1 && w > peak) {
          peak = w;
          peak_ok = fabsf(pd) <= poly_f(sg, n, sf);
        }
        if (mode == 3 && pd > 0.0f && occ == -1) occ = (float)p >= thresh;
      }
      Vprev = V;
    }
  }
  if (mode == 0) return (float)(sum / (1.0 - Vprev + (double)F_EPS_F));
  if (mode == 1) {
    if (!(d > 0.0f)) return -1.0f;
    if (any && peak > 0.0 && Vprev >= 0.9) return (s_last + poly_f(bs, n, s_last)) <= d ? -1.0f : 0.0f;
    if (any && peak > 0.0) return (float)peak_ok;
    return -1.0f;
  }
  if (mode == 2) {
    if (run_open && s_last >= d) return 0.0f;
    return -1.0f;
  }
  return (float)occ;
}

void orc_render(const orc_map* m, int mode, const float* pose, const float* depth, float thresh,
                float* out_img, int64_t* counts) {
  int H = m->p.rows, W = m->p.cols;
  float* dep = (float*)malloc((size_t)H * W * sizeof(float));
  clean_depth(&m->cam, depth, dep);
  int64_t cnt[4] = {0, 0, 0, 0};
  for (int y = 0; y < H; ++y) {
    for (int x = 0; x < W; ++x) {
      float d = dep[y * W + x];
      float v;
      if (mode != 0 && !(d > 0.0f)) v = -1.0f;
      else v = render_pixel(m, mode, pose, x, y, d, thresh);
      out_img[y * W + x] = v;
      if (mode != 0) {
        int k = (int)v + 1;
        if (k >= 0 && k < 4) cnt[k]++;
      }
    }
  }
  if (counts) memcpy(counts, cnt, sizeof(cnt));
  free(dep);
}
