/*
 * blz_oracle.c — CPU oracle for the Blitzen culling path. TEST INFRASTRUCTURE ONLY: used by the
 * tests as the checker and by the benchmark's CPU-baseline leg; the product never links it.
 * The arithmetic conventions it fixes are listed in blz_oracle.h. Build with -ffp-contract=off.
 *
 * Each function cites the reference lines it restates (paths inside the Blitzen project).
 */
#include "blz_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------ scalar conventions */

/* D3D float->uint: NaN and non-positive -> 0, >= 2^32 -> UINT32_MAX, else truncate. */
uint32_t bo_ftou(float x)
{
    if (!(x > 0.0f)) return 0u;
    if (x >= 4294967296.0f) return 0xFFFFFFFFu;
    return (uint32_t)x;
}

/* floor(log2(x)) converted to uint with the D3D rule: exact exponent for finite x >= 1. */
uint32_t bo_floor_log2_u(float x)
{
    if (!(x >= 1.0f)) return 0u;          /* x < 1, zero, negative or NaN: result <= -1 or NaN -> 0 */
    if (isinf(x)) return 0xFFFFFFFFu;     /* floor(log2(inf)) = inf -> UINT32_MAX */
    int e;
    frexpf(x, &e);                        /* x = m * 2^e, m in [0.5, 1) */
    return (uint32_t)(e - 1);
}

/* Float floor(log2(x)) for the Vulkan form (may be negative / -inf / NaN). */
static float floor_log2_f(float x)
{
    if (isnan(x) || x < 0.0f) return NAN;
    if (x == 0.0f) return -INFINITY;
    if (isinf(x)) return INFINITY;
    int e;
    frexpf(x, &e);
    return (float)(e - 1);
}

static float fmax_nan(float a, float b)     /* maxNum */
{
    if (isnan(a)) return b;
    if (isnan(b)) return a;
    return (b > a) ? b : a;
}

static float fmin_nan(float a, float b)     /* minNum, keeps a on ties */
{
    if (isnan(a)) return b;
    if (isnan(b)) return a;
    return (b < a) ? b : a;
}

/* ------------------------------------------------------------------ per-object math */

/* v + 2 * cross(q.xyz, cross(q.xyz, v) + q.w * v)
 * src/Renderer/VulkanShaderHeaders/ShaderBuffers.glsl:197-200, HlslShaders/Headers/hlslMath.hlsl:1-4 */
static void rotate_quat(const float v[3], const float q[4], float out[3])
{
    float c1x = q[1] * v[2] - q[2] * v[1];
    float c1y = q[2] * v[0] - q[0] * v[2];
    float c1z = q[0] * v[1] - q[1] * v[0];
    float tx = c1x + q[3] * v[0];
    float ty = c1y + q[3] * v[1];
    float tz = c1z + q[3] * v[2];
    float c2x = q[1] * tz - q[2] * ty;
    float c2y = q[2] * tx - q[0] * tz;
    float c2z = q[0] * ty - q[1] * tx;
    out[0] = v[0] + 2.0f * c2x;
    out[1] = v[1] + 2.0f * c2y;
    out[2] = v[2] + 2.0f * c2z;
}

/* view * vec4(p, 1), column-major, terms summed left to right (blitMLTypes.h:184-193 order). */
static void view_transform(const float m[16], const float p[3], float out[3])
{
    for (int r = 0; r < 3; ++r)
        out[r] = ((m[0 + r] * p[0] + m[4 + r] * p[1]) + m[8 + r] * p[2]) + m[12 + r] * 1.0f;
}

/* Sphere centre to world then view space: ModelSphereToViewSphere, hlslMath.hlsl:6-10;
 * IsObjectInsideViewFrustum's first lines, CullingShaderData.glsl:44-46. */
static void sphere_to_view(const float c[3], float r, const BlzMeshTransform* t, const float view[16],
                           float world[3], float vc[3], float* vr)
{
    float rot[3];
    rotate_quat(c, t->orientation, rot);
    world[0] = rot[0] * t->scale + t->pos[0];
    world[1] = rot[1] * t->scale + t->pos[1];
    world[2] = rot[2] * t->scale + t->pos[2];
    view_transform(view, world, vc);
    *vr = r * t->scale;
}

/* Symmetric side planes, then near/far on view z. hlslMath.hlsl:13-27, CullingShaderData.glsl:52-55 */
static int frustum_check(const float c[3], float r, const BlzCameraViewData* v)
{
    int visible = 1;
    visible = visible && (c[2] * v->frustumLeft - fabsf(c[0]) * v->frustumRight > -r);
    visible = visible && (c[2] * v->frustumBottom - fabsf(c[1]) * v->frustumTop > -r);
    visible = visible && (c[2] + r > v->zNear) && (c[2] - r < v->zFar);
    return visible;
}

/* Mara & McGuire 2013 projected-sphere bounds in UV space.
 * hlslMath.hlsl:30-56 (ProjectSphere), CullingShaderData.glsl:8-33 (projectSphere). */
static int project_sphere(const float c[3], float r, float znear, float P00, float P11, float aabb[4])
{
    if (c[2] < r + znear) return 0;
    float sx = c[0] * r, sy = c[1] * r, sz = c[2] * r;
    float zp = c[2] * c[2] - r * r;
    float xr = sqrtf(c[0] * c[0] + zp);
    float xmin = (xr * c[0] - sz) / (xr * c[2] + sx);
    float xmax = (xr * c[0] + sz) / (xr * c[2] - sx);
    float yr = sqrtf(c[1] * c[1] + zp);
    float ymin = (yr * c[1] - sz) / (yr * c[2] + sy);
    float ymax = (yr * c[1] + sz) / (yr * c[2] - sy);
    float a0 = xmin * P00, a1 = ymin * P11, a2 = xmax * P00, a3 = ymax * P11;
    /* aabb.xwzy * (0.5, -0.5, 0.5, -0.5) + 0.5 */
    aabb[0] = a0 * 0.5f + 0.5f;
    aabb[1] = a3 * -0.5f + 0.5f;
    aabb[2] = a2 * 0.5f + 0.5f;
    aabb[3] = a1 * -0.5f + 0.5f;
    return 1;
}

static float pyr_load(const BlzPyramid* p, uint32_t level, uint32_t x, uint32_t y)
{
    if (level >= p->mipCount) return 0.0f;
    uint32_t w = p->width >> level, h = p->height >> level;
    if (w < 1) w = 1;
    if (h < 1) h = 1;
    if (x >= w || y >= h) return 0.0f;
    return p->data[p->mipOffset[level] + (uint64_t)y * w + x];
}

/* D3D12 occlusion test: one-texel Load at the footprint centre of mip floor(log2(size)).
 * hlslMath.hlsl:58-78 (OcclusionCheck). */
static int occlusion_d3d12(const float aabb_in[4], const BlzPyramid* p, const BlzCameraViewData* v,
                           const float c[3], float r)
{
    uint32_t pw = bo_ftou(v->pyramidWidth);   /* float constant passed to a uint parameter */
    uint32_t ph = bo_ftou(v->pyramidHeight);
    float a[4] = {aabb_in[0], aabb_in[1], aabb_in[2], aabb_in[3]};
    float width = (a[2] - a[0]) * (float)pw;
    float height = (a[3] - a[1]) * (float)ph;
    uint32_t level = bo_floor_log2_u(fmax_nan(width, height));
    float depth = 0.0f;
    if (level < p->mipCount) {
        uint32_t mw = pw >> level, mh = ph >> level;
        if (mw < 1u) mw = 1u;
        if (mh < 1u) mh = 1u;
        float sw = (float)mw * 0.5f, sh = (float)mh * 0.5f;
        a[0] *= sw;
        a[1] *= sh;
        a[2] *= sw;
        a[3] *= sh;
        depth = pyr_load(p, level, bo_ftou(a[0] + a[2]), bo_ftou(a[1] + a[3]));
    }
    float depthSphere = v->zNear / (c[2] - r);
    return depthSphere > depth;
}

/* MIN-reduction bilinear footprint at normalised (s, t) in one mip, clamp-to-edge: the texels
 * with non-zero weight are i0 = floor(s*W - 0.5) and, when the fraction is > 0, i0 + 1; same in y.
 * Sampler of src/Renderer/BlitzenVulkan/vulkanResources.cpp:51-55 (LINEAR, MIN, CLAMP_TO_EDGE). */
static int64_t to_index(float f)   /* NaN -> 0; huge magnitudes saturate before the edge clamp */
{
    if (isnan(f)) return 0;
    if (f < -1.0e18f) return -((int64_t)1 << 60);
    if (f > 1.0e18f) return (int64_t)1 << 60;
    return (int64_t)f;
}

static float min_footprint(const float* img, uint32_t w, uint32_t h, float s, float t)
{
    float u = s * (float)w - 0.5f, vv = t * (float)h - 0.5f;
    float fu = floorf(u), fv = floorf(vv);
    float au = u - fu, av = vv - fv;
    int64_t i0 = to_index(fu), j0 = to_index(fv);
    int64_t i1 = (au > 0.0f) ? i0 + 1 : i0;
    int64_t j1 = (av > 0.0f) ? j0 + 1 : j0;
    int64_t xs[2] = {i0, i1}, ys[2] = {j0, j1};
    float m = NAN;
    for (int jy = 0; jy < 2; ++jy)
        for (int ix = 0; ix < 2; ++ix) {
            int64_t x = xs[ix], y = ys[jy];
            if (x < 0) x = 0;
            if (x > (int64_t)w - 1) x = (int64_t)w - 1;
            if (y < 0) y = 0;
            if (y > (int64_t)h - 1) y = (int64_t)h - 1;
            m = fmin_nan(m, img[(uint64_t)y * w + (uint64_t)x]);
        }
    return m;
}

static uint32_t vk_mip_select(float level, uint32_t mipCount)
{
    /* lambda = clamp(level, minLod 0, maxLod 16), NEAREST mip of integer lambda, clamp to last mip */
    float lam = level;
    if (!(lam > 0.0f)) lam = 0.0f;
    if (lam > 16.0f) lam = 16.0f;
    uint32_t d = (uint32_t)lam;
    if (d > mipCount - 1u) d = mipCount - 1u;
    return d;
}

/* Vulkan occlusion test: textureLod at the footprint centre with the MIN sampler.
 * CullingShaderData.glsl:60-73 (OcclusionCullingPassed). */
static int occlusion_vulkan(const float a[4], const BlzPyramid* p, const BlzCameraViewData* v,
                            const float c[3], float r)
{
    float width = (a[2] - a[0]) * v->pyramidWidth;
    float height = (a[3] - a[1]) * v->pyramidHeight;
    float level = floor_log2_f(fmax_nan(width, height));
    uint32_t d = vk_mip_select(level, p->mipCount);
    uint32_t w = p->width >> d, h = p->height >> d;
    if (w < 1) w = 1;
    if (h < 1) h = 1;
    float s = (a[0] + a[2]) * 0.5f, t = (a[1] + a[3]) * 0.5f;
    float depth = min_footprint(p->data + p->mipOffset[d], w, h, s, t);
    float depthSphere = v->zNear / (c[2] - r);
    return depthSphere > depth;
}

static int occlusion(const float aabb[4], const BlzPyramid* p, const BlzCameraViewData* v, const float c[3], float r)
{
    return (p->mode == BLZ_HIZ_VULKAN) ? occlusion_vulkan(aabb, p, v, c, r) : occlusion_d3d12(aabb, p, v, c, r);
}

/* Last LOD in [1, lodCount) whose error is below distance * lodTarget / scale, else 0.
 * CullingShaderData.glsl:103-116, HlslShaders/Headers/cullBuffers.hlsl:42-55. */
static uint32_t lod_select(const float c[3], float r, float scale, float lodTarget, const BlzLodData* lods,
                           uint32_t lodOffset, uint32_t lodCount)
{
    float len = sqrtf((c[0] * c[0] + c[1] * c[1]) + c[2] * c[2]);
    float d = len - r;
    float distance = (d > 0.0f) ? d : 0.0f;
    float threshold = distance * lodTarget / scale;
    uint32_t idx = 0;
    for (uint32_t i = 1; i < lodCount; ++i)
        if (lods[lodOffset + i].error < threshold) idx = i;
    return lodOffset + idx;
}

typedef struct {
    float world[3], vc[3], vr;
    const BlzMeshTransform* t;
    const BlzPrimitiveSurface* s;
} ObjState;

/* Table lookups with range checks (the reference reads past the end; we refuse and flag). */
static int fetch_object(const BlzSceneDesc* sc, BlzRenderObject o, const float view[16], ObjState* st)
{
    if (o.transformId >= sc->transformCount || o.surfaceId >= sc->surfaceCount) return 0;
    st->t = &sc->transforms[o.transformId];
    st->s = &sc->surfaces[o.surfaceId];
    if (st->s->lodOffset >= sc->lodCount || st->s->lodCount > sc->lodCount - st->s->lodOffset) return 0;
    sphere_to_view(st->s->center, st->s->radius, st->t, view, st->world, st->vc, &st->vr);
    return 1;
}

/* Visibility decision of one object for a mode: drawCull / drawOccFirst (frustum), drawOccLate /
 * drawOccTemporal (frustum, then projectSphere + Hi-Z when the sphere is in front of near).
 * Returns 1 visible, 0 culled, -1 bad index. */
static int object_visible(int mode, const BlzCameraViewData* v, const BlzSceneDesc* sc, BlzRenderObject o,
                          const BlzPyramid* p, ObjState* st)
{
    if (!fetch_object(sc, o, v->viewMatrix, st)) return -1;
    int visible = frustum_check(st->vc, st->vr, v);
    if ((mode == BO_LATE || mode == BO_TEMPORAL) && visible) {
        float aabb[4];
        if (project_sphere(st->vc, st->vr, v->zNear, v->proj0, v->proj5, aabb))
            visible = visible && occlusion(aabb, p, v, st->vc, st->vr);
    }
    return visible;
}

int bo_object_test(int mode, const BlzCameraViewData* view, const BlzSceneDesc* scene, BlzRenderObject obj,
                   const BlzPyramid* pyramid, uint32_t* lodIdOut)
{
    ObjState st;
    int vis = object_visible(mode, view, scene, obj, pyramid, &st);
    if (vis > 0 && lodIdOut)
        *lodIdOut = lod_select(st.vc, st.vr, st.t->scale, view->lodTarget, scene->lods, st.s->lodOffset, st.s->lodCount);
    return vis;
}

static void put_record(void* cmds, uint32_t stride, uint32_t slot, uint32_t a, uint32_t b, uint32_t c, uint32_t d)
{
    uint32_t* w = (uint32_t*)((char*)cmds + (uint64_t)slot * stride);
    w[0] = a;  /* objectId / objId */
    w[1] = b;  /* indexCount */
    w[2] = c;  /* instanceCount */
    w[3] = d;  /* firstIndex */
    w[4] = 0;  /* vertexOffset */
    w[5] = 0;  /* firstInstance */
}

/* ------------------------------------------------------------------ range workers */

typedef struct {
    /* inputs */
    int kind;               /* 0 object cull, 1 instanced, 2 clusters */
    int mode;
    const BlzCameraViewData* view;
    const BlzSceneDesc* scene;
    const BlzRenderObject* objects;
    uint32_t begin, end;
    uint32_t* vis;
    const BlzPyramid* pyramid;
    /* outputs: local record list (6 words each) and optional cluster ids / instance lod ids */
    uint32_t* rec;
    uint32_t* ids;
    uint32_t n, cap;
    uint32_t flags;
} Work;

static void work_push(Work* w, uint32_t a, uint32_t b, uint32_t c, uint32_t d, uint32_t id)
{
    if (w->n == w->cap) {
        uint32_t ncap = w->cap ? w->cap * 2 : 1024;
        w->rec = (uint32_t*)realloc(w->rec, (size_t)ncap * 4 * sizeof(uint32_t));
        w->ids = (uint32_t*)realloc(w->ids, (size_t)ncap * sizeof(uint32_t));
        w->cap = ncap;
    }
    uint32_t* r = w->rec + (size_t)w->n * 4;
    r[0] = a; r[1] = b; r[2] = c; r[3] = d;
    w->ids[w->n] = id;
    w->n++;
}

/* drawCull / drawOccFirst / drawOccLate / drawOccTemporal bodies (HlslShaders/CS/*.cs.hlsl),
 * InitialDrawCull / LateDrawCull / TransparentDrawCull (VulkanShaders). */
static void range_objects(Work* w)
{
    const BlzSceneDesc* sc = w->scene;
    for (uint32_t i = w->begin; i < w->end; ++i) {
        if (w->mode == BO_FIRST && w->vis[i] == 0) continue;   /* drawOccFirst.cs.hlsl:22-25 */
        ObjState st;
        int visible = object_visible(w->mode, w->view, sc, w->objects[i], w->pyramid, &st);
        if (visible < 0) { w->flags |= BLZ_FLAG_BAD_INDEX; visible = 0; }
        int emit = visible;
        if (w->mode == BO_LATE) emit = visible && w->vis[i] == 0; /* drawOccLate.cs.hlsl:45 */
        if (emit) {
            uint32_t lodId = lod_select(st.vc, st.vr, st.t->scale, w->view->lodTarget, sc->lods,
                                        st.s->lodOffset, st.s->lodCount);
            const BlzLodData* L = &sc->lods[lodId];
            work_push(w, i, L->indexCount, 1u, L->firstIndex, lodId);
        }
        if (w->mode == BO_LATE) w->vis[i] = visible ? 1u : 0u;  /* drawOccLate.cs.hlsl:67 */
    }
}

/* drawInstCull.cs.hlsl:12-42 body: record (objId, lodId) of each visible object. */
static void range_instanced(Work* w)
{
    const BlzSceneDesc* sc = w->scene;
    for (uint32_t i = w->begin; i < w->end; ++i) {
        ObjState st;
        int visible = object_visible(BO_FRUSTUM, w->view, sc, w->objects[i], NULL, &st);
        if (visible < 0) { w->flags |= BLZ_FLAG_BAD_INDEX; continue; }
        if (!visible) continue;
        uint32_t lodId = lod_select(st.vc, st.vr, st.t->scale, w->view->lodTarget, sc->lods,
                                    st.s->lodOffset, st.s->lodCount);
        work_push(w, i, lodId, 0, 0, lodId);
    }
}

/* Cluster path: PreClusterDrawCull.comp.glsl:13-47 (object frustum + LOD, expansion over the LOD's
 * clusters) fused with the per-cluster tests the reference leaves commented out
 * (InitialClusterCull.comp.glsl:24-42): sphere frustum, Hi-Z, and the normal-cone test in
 * meshoptimizer's documented form, cull when dot(normalize(center - camera), axis) >= cutoff
 * (VendorCode/Meshoptimizer/meshoptimizer.h:561-569). Emits InitialClusterCull.comp.glsl:48-54. */
static void range_clusters(Work* w)
{
    const BlzSceneDesc* sc = w->scene;
    const BlzCameraViewData* v = w->view;
    for (uint32_t i = w->begin; i < w->end; ++i) {
        ObjState st;
        int visible = object_visible(BO_FRUSTUM, v, sc, w->objects[i], NULL, &st);
        if (visible < 0) { w->flags |= BLZ_FLAG_BAD_INDEX; continue; }
        if (!visible) continue;
        uint32_t lodId = lod_select(st.vc, st.vr, st.t->scale, v->lodTarget, sc->lods, st.s->lodOffset, st.s->lodCount);
        const BlzLodData* L = &sc->lods[lodId];
        if (L->clusterOffset > sc->clusterCount || L->clusterCount > sc->clusterCount - L->clusterOffset) {
            w->flags |= BLZ_FLAG_BAD_INDEX;
            continue;
        }
        for (uint32_t k = 0; k < L->clusterCount; ++k) {
            uint32_t cid = L->clusterOffset + k;
            const BlzCluster* cl = &sc->clusters[cid];
            float world[3], vc[3], vr;
            sphere_to_view(cl->center, cl->radius, st.t, v->viewMatrix, world, vc, &vr);
            int vis = frustum_check(vc, vr, v);
            if (vis && w->pyramid) {
                float aabb[4];
                if (project_sphere(vc, vr, v->zNear, v->proj0, v->proj5, aabb))
                    vis = vis && occlusion(aabb, w->pyramid, v, vc, vr);
            }
            if (vis) {
                float axm[3] = {(float)cl->coneAxisX / 127.0f, (float)cl->coneAxisY / 127.0f,
                                (float)cl->coneAxisZ / 127.0f};
                float cutoff = (float)cl->coneCutoff / 127.0f;
                float axis[3];
                rotate_quat(axm, st.t->orientation, axis);
                float dx = world[0] - v->position[0], dy = world[1] - v->position[1], dz = world[2] - v->position[2];
                float len = sqrtf((dx * dx + dy * dy) + dz * dz);
                float nx = dx / len, ny = dy / len, nz = dz / len;
                float dp = (nx * axis[0] + ny * axis[1]) + nz * axis[2];
                if (dp >= cutoff) vis = 0;
            }
            if (vis) work_push(w, i, (uint32_t)cl->triangleCount * 3u, 1u, cl->dataOffset, cid);
        }
    }
}

static void* work_thread(void* arg)
{
    Work* w = (Work*)arg;
    if (w->kind == 0) range_objects(w);
    else if (w->kind == 1) range_instanced(w);
    else range_clusters(w);
    return NULL;
}

/* Splits [0, count) into `threads` contiguous ranges and runs them; results stay per range. */
static Work* run_ranges(Work proto, uint32_t count, int threads)
{
    if (threads < 1) threads = 1;
    if ((uint32_t)threads > count) threads = count ? (int)count : 1;
    Work* ws = (Work*)calloc((size_t)threads + 1, sizeof(Work));
    uint32_t per = count / (uint32_t)threads, rem = count % (uint32_t)threads, at = 0;
    for (int t = 0; t < threads; ++t) {
        ws[t] = proto;
        ws[t].begin = at;
        at += per + ((uint32_t)t < rem ? 1u : 0u);
        ws[t].end = at;
        ws[t].rec = NULL; ws[t].ids = NULL; ws[t].n = ws[t].cap = 0; ws[t].flags = 0;
    }
    ws[threads].kind = -1; /* terminator */
    if (threads == 1) {
        work_thread(&ws[0]);
    } else {
        pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * (size_t)threads);
        for (int t = 0; t < threads; ++t) pthread_create(&th[t], NULL, work_thread, &ws[t]);
        for (int t = 0; t < threads; ++t) pthread_join(th[t], NULL);
        free(th);
    }
    return ws;
}

static void free_ranges(Work* ws)
{
    for (int t = 0; ws[t].kind != -1; ++t) { free(ws[t].rec); free(ws[t].ids); }
    free(ws);
}

/* ------------------------------------------------------------------ public culls */

uint32_t bo_cull(int mode, const BlzCameraViewData* view, const BlzSceneDesc* scene, const BlzRenderObject* objects,
                 uint32_t count, uint32_t* vis, const BlzPyramid* pyramid, void* cmds, uint32_t stride,
                 uint32_t capacity, uint32_t* flags, int threads)
{
    Work proto;
    memset(&proto, 0, sizeof proto);
    proto.kind = 0; proto.mode = mode; proto.view = view; proto.scene = scene;
    proto.objects = objects ? objects : scene->renderObjects;
    proto.vis = vis; proto.pyramid = pyramid;
    Work* ws = run_ranges(proto, count, threads);
    uint32_t total = 0, f = 0;
    for (int t = 0; ws[t].kind != -1; ++t) {
        f |= ws[t].flags;
        for (uint32_t k = 0; k < ws[t].n; ++k, ++total) {
            if (total < capacity) {
                const uint32_t* r = ws[t].rec + (size_t)k * 4;
                put_record(cmds, stride, total, r[0], r[1], r[2], r[3]);
            }
        }
    }
    if (total > capacity) f |= BLZ_FLAG_COMMAND_OVERFLOW;
    free_ranges(ws);
    if (flags) *flags |= f;
    return total;
}

/* drawInstCountReset.cs.hlsl:9-18, drawInstCull.cs.hlsl:38-41, drawInstCmd.cs.hlsl:9-38. */
uint32_t bo_cull_instanced(const BlzCameraViewData* view, const BlzSceneDesc* scene, const BlzRenderObject* objects,
                           uint32_t count, BlzLodInstanceCounter* counters, uint32_t* instances,
                           uint32_t instanceCapacity, uint32_t slotsPerLod, void* cmds, uint32_t stride,
                           uint32_t capacity, uint32_t* flags, int threads)
{
    uint32_t f = 0;
    uint32_t slots = slotsPerLod ? slotsPerLod : 0xFFFFFFFFu;
    for (uint32_t l = 0; l < scene->lodCount; ++l) counters[l].instanceCount = 0;
    Work proto;
    memset(&proto, 0, sizeof proto);
    proto.kind = 1; proto.view = view; proto.scene = scene;
    proto.objects = objects ? objects : scene->renderObjects;
    Work* ws = run_ranges(proto, count, threads);
    for (int t = 0; ws[t].kind != -1; ++t) {
        f |= ws[t].flags;
        for (uint32_t k = 0; k < ws[t].n; ++k) {
            uint32_t obj = ws[t].rec[(size_t)k * 4], lod = ws[t].rec[(size_t)k * 4 + 1];
            uint32_t slot = counters[lod].instanceCount++;
            uint64_t at = (uint64_t)counters[lod].instanceOffset + slot;
            if (slot < slots && at < instanceCapacity) instances[at] = obj;
            else f |= BLZ_FLAG_INSTANCE_OVERFLOW;
        }
    }
    free_ranges(ws);
    uint32_t n = 0;
    for (uint32_t l = 0; l < scene->lodCount; ++l) {
        uint32_t c = counters[l].instanceCount;
        if (c == 0) continue;
        if (n < capacity) {
            uint32_t shown = c < slots ? c : slots;
            put_record(cmds, stride, n, counters[l].instanceOffset, scene->lods[l].indexCount, shown,
                       scene->lods[l].firstIndex);
        }
        n++;
    }
    if (n > capacity) f |= BLZ_FLAG_COMMAND_OVERFLOW;
    if (flags) *flags |= f;
    return n;
}

uint32_t bo_cull_clusters(const BlzCameraViewData* view, const BlzSceneDesc* scene, const BlzRenderObject* objects,
                          uint32_t count, const BlzPyramid* pyramid, void* cmds, uint32_t stride, uint32_t capacity,
                          uint32_t* clusterIds, uint32_t* flags, int threads)
{
    Work proto;
    memset(&proto, 0, sizeof proto);
    proto.kind = 2; proto.view = view; proto.scene = scene;
    proto.objects = objects ? objects : scene->renderObjects;
    proto.pyramid = pyramid;
    Work* ws = run_ranges(proto, count, threads);
    uint32_t total = 0, f = 0;
    for (int t = 0; ws[t].kind != -1; ++t) {
        f |= ws[t].flags;
        for (uint32_t k = 0; k < ws[t].n; ++k, ++total) {
            if (total < capacity) {
                const uint32_t* r = ws[t].rec + (size_t)k * 4;
                put_record(cmds, stride, total, r[0], r[1], r[2], r[3]);
                if (clusterIds) clusterIds[total] = ws[t].ids[k];
            }
        }
    }
    if (total > capacity) f |= BLZ_FLAG_COMMAND_OVERFLOW;
    free_ranges(ws);
    if (flags) *flags |= f;
    return total;
}

/* ------------------------------------------------------------------ depth pyramid */

static uint32_t mip_levels(uint32_t w, uint32_t h)   /* blitML.h:95-107 */
{
    uint32_t n = 0;
    while (w > 1 || h > 1) { n++; w /= 2; h /= 2; }
    return n;
}

static uint32_t prev_pow2(uint32_t v)                /* blitML.h:54-62 */
{
    uint32_t r = 1;
    while (r * 2 < v) r *= 2;
    return r;
}

uint64_t bo_pyramid_layout(uint32_t dw, uint32_t dh, uint32_t mode, BlzPyramid* out)
{
    if (!out || dw == 0 || dh == 0 || mode > BLZ_HIZ_VULKAN) return 0;
    memset(out, 0, sizeof *out);
    out->mode = mode;
    out->depthWidth = dw;
    out->depthHeight = dh;
    if (mode == BLZ_HIZ_D3D12) {       /* dx12RNDResources.cpp:103-106 */
        out->width = (dw >> 1) ? (dw >> 1) : 1;
        out->height = (dh >> 1) ? (dh >> 1) : 1;
    } else {                           /* vulkanResources.cpp:93-95 */
        out->width = prev_pow2(dw);
        out->height = prev_pow2(dh);
    }
    uint32_t n = mip_levels(out->width, out->height);
    if (n == 0) n = 1;                 /* a 1x1 pyramid still has its one level */
    if (n > BLZ_PYRAMID_MAX_MIPS) return 0;
    out->mipCount = n;
    uint64_t at = 0;
    for (uint32_t i = 0; i < n; ++i) {
        uint32_t w = out->width >> i, h = out->height >> i;
        if (w < 1) w = 1;
        if (h < 1) h = 1;
        out->mipOffset[i] = (uint32_t)at;
        at += (uint64_t)w * h;
    }
    return at * sizeof(float);
}

/* depthPyramid.cs.hlsl:13-26 dispatched per mip as in dx12Draw.cpp:248-277: level 0 reads the depth
 * target at mip 0, level i reads pyramid mip i-1; each texel is min(r, min(g, min(b, a))) of the
 * 2x2 Loads at (2x,2y), (2x+1,2y), (2x,2y+1), (2x+1,2y+1); out-of-range Loads give 0. */
static void build_d3d12(const BlzPyramid* p, const float* depth)
{
    for (uint32_t i = 0; i < p->mipCount; ++i) {
        uint32_t w = p->width >> i, h = p->height >> i;
        if (w < 1) w = 1;
        if (h < 1) h = 1;
        const float* src;
        uint32_t sw, sh;
        if (i == 0) { src = depth; sw = p->depthWidth; sh = p->depthHeight; }
        else {
            src = p->data + p->mipOffset[i - 1];
            sw = p->width >> (i - 1); sh = p->height >> (i - 1);
            if (sw < 1) sw = 1;
            if (sh < 1) sh = 1;
        }
        float* dst = p->data + p->mipOffset[i];
        for (uint32_t y = 0; y < h; ++y)
            for (uint32_t x = 0; x < w; ++x) {
                uint64_t x0 = 2ull * x, y0 = 2ull * y;
                float r = (x0 < sw && y0 < sh) ? src[y0 * sw + x0] : 0.0f;
                float g = (x0 + 1 < sw && y0 < sh) ? src[y0 * sw + x0 + 1] : 0.0f;
                float b = (x0 < sw && y0 + 1 < sh) ? src[(y0 + 1) * sw + x0] : 0.0f;
                float a = (x0 + 1 < sw && y0 + 1 < sh) ? src[(y0 + 1) * sw + x0 + 1] : 0.0f;
                dst[(uint64_t)y * w + x] = fmin_nan(r, fmin_nan(g, fmin_nan(b, a)));
            }
    }
}

/* DepthPyramidGeneration.comp.glsl:13-19 per mip as in vulkanDraw.cpp:579-614: texel (x, y) of mip i
 * samples the previous level (the depth attachment for i = 0) at ((x + 0.5) / w_i, (y + 0.5) / h_i)
 * with the MIN-reduction bilinear sampler. */
static void build_vulkan(const BlzPyramid* p, const float* depth)
{
    for (uint32_t i = 0; i < p->mipCount; ++i) {
        uint32_t w = p->width >> i, h = p->height >> i;
        if (w < 1) w = 1;
        if (h < 1) h = 1;
        const float* src;
        uint32_t sw, sh;
        if (i == 0) { src = depth; sw = p->depthWidth; sh = p->depthHeight; }
        else {
            src = p->data + p->mipOffset[i - 1];
            sw = p->width >> (i - 1); sh = p->height >> (i - 1);
            if (sw < 1) sw = 1;
            if (sh < 1) sh = 1;
        }
        float* dst = p->data + p->mipOffset[i];
        float fw = (float)w, fh = (float)h;
        for (uint32_t y = 0; y < h; ++y)
            for (uint32_t x = 0; x < w; ++x) {
                float s = ((float)x + 0.5f) / fw, t = ((float)y + 0.5f) / fh;
                dst[(uint64_t)y * w + x] = min_footprint(src, sw, sh, s, t);
            }
    }
}

void bo_pyramid_build(const BlzPyramid* p, const float* depth)
{
    if (p->mode == BLZ_HIZ_VULKAN) build_vulkan(p, depth);
    else build_d3d12(p, depth);
}

/* ------------------------------------------------------------------ transforms */

void bo_transforms_update(BlzMeshTransform* table, uint32_t tableCount, const uint32_t* ids,
                          const BlzMeshTransform* in, uint32_t n, uint32_t* flags)
{
    for (uint32_t i = 0; i < n; ++i) {
        if (ids[i] >= tableCount) { if (flags) *flags |= BLZ_FLAG_BAD_INDEX; continue; }
        table[ids[i]] = in[i];
    }
}

/* q' = r (x) q with r = (sin(a/2) * axis, cos(a/2)); Hamilton product written out. */
void bo_transforms_rotate(const BlzMeshTransform* table, uint32_t tableCount, const uint32_t* ids,
                          const float* axes, float angle, uint32_t n, BlzMeshTransform* dst, uint32_t* flags)
{
    float h = angle * 0.5f;
    float s = sinf(h), c = cosf(h);
    for (uint32_t i = 0; i < n; ++i) {
        if (ids[i] >= tableCount) { if (flags) *flags |= BLZ_FLAG_BAD_INDEX; continue; }
        BlzMeshTransform t = table[ids[i]];
        float rx = s * axes[3 * i + 0], ry = s * axes[3 * i + 1], rz = s * axes[3 * i + 2], rw = c;
        float qx = t.orientation[0], qy = t.orientation[1], qz = t.orientation[2], qw = t.orientation[3];
        t.orientation[0] = ((rw * qx + rx * qw) + ry * qz) - rz * qy;
        t.orientation[1] = ((rw * qy - rx * qz) + ry * qw) + rz * qx;
        t.orientation[2] = ((rw * qz + rx * qy) - ry * qx) + rz * qw;
        t.orientation[3] = ((rw * qw - rx * qx) - ry * qy) - rz * qz;
        dst[i] = t;
    }
}

/* ------------------------------------------------------------------ occluder raster */

void bo_depth_raster_boxes(const BlzCameraViewData* v, const float* boxes, uint32_t boxCount, float* depth,
                           uint32_t width, uint32_t height)
{
    memset(depth, 0, sizeof(float) * (size_t)width * height);
    float fw = (float)width, fh = (float)height;
    for (uint32_t b = 0; b < boxCount; ++b) {
        const float* bx = boxes + 6 * (size_t)b;
        float minx = INFINITY, maxx = -INFINITY, miny = INFINITY, maxy = -INFINITY, zmax = -INFINITY;
        int ok = 1;
        for (int k = 0; k < 8; ++k) {
            float p[3] = {bx[(k & 1) ? 3 : 0], bx[(k & 2) ? 4 : 1], bx[(k & 4) ? 5 : 2]};
            float q[3];
            view_transform(v->viewMatrix, p, q);
            if (!(q[2] > v->zNear)) { ok = 0; break; }
            float sx = ((q[0] * v->proj0) / q[2] * 0.5f + 0.5f) * fw;
            float sy = (0.5f - (q[1] * v->proj5) / q[2] * 0.5f) * fh;
            minx = fminf(minx, sx); maxx = fmaxf(maxx, sx);
            miny = fminf(miny, sy); maxy = fmaxf(maxy, sy);
            zmax = fmaxf(zmax, q[2]);
        }
        if (!ok) continue;
        float d = v->zNear / zmax;
        float fx0 = floorf(minx), fy0 = floorf(miny), fx1 = ceilf(maxx), fy1 = ceilf(maxy);
        int64_t x0 = fx0 < 0.0f ? 0 : (fx0 > fw ? (int64_t)width : (int64_t)fx0);
        int64_t y0 = fy0 < 0.0f ? 0 : (fy0 > fh ? (int64_t)height : (int64_t)fy0);
        int64_t x1 = fx1 < 0.0f ? 0 : (fx1 > fw ? (int64_t)width : (int64_t)fx1);
        int64_t y1 = fy1 < 0.0f ? 0 : (fy1 > fh ? (int64_t)height : (int64_t)fy1);
        for (int64_t y = y0; y < y1; ++y)
            for (int64_t x = x0; x < x1; ++x) {
                float* px = &depth[(size_t)y * width + (size_t)x];
                if (d > *px) *px = d;
            }
    }
}

/* ------------------------------------------------------------------ view constants */

typedef struct { float m[16]; } M4;

static M4 m4_identity(void) { M4 r; memset(&r, 0, sizeof r); r.m[0] = r.m[5] = r.m[10] = r.m[15] = 1.0f; return r; }

/* blitMLTypes.h:172-182: res[j + i*4] = sum_k a[4k + j] * b[k + i*4], summed left to right. */
static M4 m4_mul(const M4* a, const M4* b)
{
    M4 r;
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j)
            r.m[j + i * 4] = ((a->m[0 + j] * b->m[0 + i * 4] + a->m[4 + j] * b->m[1 + i * 4]) +
                              a->m[8 + j] * b->m[2 + i * 4]) + a->m[12 + j] * b->m[3 + i * 4];
    return r;
}

/* Cofactor inverse with the same products and sums as Mat4Inverse (blitML.h:312-363). */
static M4 m4_inverse(const M4* src)
{
    const float* m = src->m;
    float p[24];
    static const int A[24][2] = {{10,15},{14,11},{6,15},{14,7},{6,11},{10,7},{2,15},{14,3},{2,11},{10,3},{2,7},{6,3},
                                 {8,13},{12,9},{4,13},{12,5},{4,9},{8,5},{0,13},{12,1},{0,9},{8,1},{0,5},{4,1}};
    for (int k = 0; k < 24; ++k) p[k] = m[A[k][0]] * m[A[k][1]];
    M4 r;
    float* o = r.m;
    o[0] = (p[0] * m[5] + p[3] * m[9] + p[4] * m[13]) - (p[1] * m[5] + p[2] * m[9] + p[5] * m[13]);
    o[1] = (p[1] * m[1] + p[6] * m[9] + p[9] * m[13]) - (p[0] * m[1] + p[7] * m[9] + p[8] * m[13]);
    o[2] = (p[2] * m[1] + p[7] * m[5] + p[10] * m[13]) - (p[3] * m[1] + p[6] * m[5] + p[11] * m[13]);
    o[3] = (p[5] * m[1] + p[8] * m[5] + p[11] * m[9]) - (p[4] * m[1] + p[9] * m[5] + p[10] * m[9]);
    float d = 1.0f / (m[0] * o[0] + m[4] * o[1] + m[8] * o[2] + m[12] * o[3]);
    o[0] = d * o[0];
    o[1] = d * o[1];
    o[2] = d * o[2];
    o[3] = d * o[3];
    o[4] = d * ((p[1] * m[4] + p[2] * m[8] + p[5] * m[12]) - (p[0] * m[4] + p[3] * m[8] + p[4] * m[12]));
    o[5] = d * ((p[0] * m[0] + p[7] * m[8] + p[8] * m[12]) - (p[1] * m[0] + p[6] * m[8] + p[9] * m[12]));
    o[6] = d * ((p[3] * m[0] + p[6] * m[4] + p[11] * m[12]) - (p[2] * m[0] + p[7] * m[4] + p[10] * m[12]));
    o[7] = d * ((p[4] * m[0] + p[9] * m[4] + p[10] * m[8]) - (p[5] * m[0] + p[8] * m[4] + p[11] * m[8]));
    o[8] = d * ((p[12] * m[7] + p[15] * m[11] + p[16] * m[15]) - (p[13] * m[7] + p[14] * m[11] + p[17] * m[15]));
    o[9] = d * ((p[13] * m[3] + p[18] * m[11] + p[21] * m[15]) - (p[12] * m[3] + p[19] * m[11] + p[20] * m[15]));
    o[10] = d * ((p[14] * m[3] + p[19] * m[7] + p[22] * m[15]) - (p[15] * m[3] + p[18] * m[7] + p[23] * m[15]));
    o[11] = d * ((p[17] * m[3] + p[20] * m[7] + p[23] * m[11]) - (p[16] * m[3] + p[21] * m[7] + p[22] * m[11]));
    o[12] = d * ((p[14] * m[10] + p[17] * m[14] + p[13] * m[6]) - (p[16] * m[14] + p[12] * m[6] + p[15] * m[10]));
    o[13] = d * ((p[20] * m[14] + p[12] * m[2] + p[19] * m[10]) - (p[18] * m[10] + p[21] * m[14] + p[13] * m[2]));
    o[14] = d * ((p[18] * m[6] + p[23] * m[14] + p[15] * m[2]) - (p[22] * m[14] + p[14] * m[2] + p[19] * m[6]));
    o[15] = d * ((p[22] * m[10] + p[16] * m[2] + p[21] * m[6]) - (p[20] * m[6] + p[23] * m[10] + p[17] * m[2]));
    return r;
}

/* QuatToMat4 (blitML.h:520-534) with NormalizeQuat (blitML.h:497-502). */
static M4 quat_to_m4(const float q[4])
{
    float nrm = sqrtf(q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3]);
    float x = q[0] / nrm, y = q[1] / nrm, z = q[2] / nrm, w = q[3] / nrm;
    M4 r = m4_identity();
    r.m[0] = 1.0f - 2.0f * y * y - 2.0f * z * z;
    r.m[1] = 2.0f * x * y - 2.0f * z * w;
    r.m[2] = 2.0f * x * z + 2.0f * y * w;
    r.m[4] = 2.0f * x * y + 2.0f * z * w;
    r.m[5] = 1.0f - 2.0f * x * x - 2.0f * z * z;
    r.m[6] = 2.0f * y * z - 2.0f * x * w;
    r.m[8] = 2.0f * x * z - 2.0f * y * w;
    r.m[9] = 2.0f * y * z + 2.0f * x * w;
    r.m[10] = 1.0f - 2.0f * x * x - 2.0f * y * y;
    return r;
}

/* QuatFromAngleAxis without normalisation (blitML.h:559-570). */
static void quat_angle_axis(float ax, float ay, float az, float angle, float q[4])
{
    float h = 0.5f * angle;
    float s = sinf(h), c = cosf(h);
    q[0] = s * ax; q[1] = s * ay; q[2] = s * az; q[3] = c;
}

void bo_view_setup(BlzCameraViewData* out, float fov, float ww, float wh, float zNear, float zFar,
                   const float pos[3], float yaw, float pitch, float pyrW, float pyrH)
{
    memset(out, 0, sizeof *out);
    out->zNear = zNear;
    out->zFar = zFar;
    out->position[0] = pos[0]; out->position[1] = pos[1]; out->position[2] = pos[2];
    M4 tr = m4_identity();
    tr.m[12] = pos[0]; tr.m[13] = pos[1]; tr.m[14] = pos[2];
    float qy[4], qp[4];
    quat_angle_axis(0.0f, -1.0f, 0.0f, yaw, qy);
    quat_angle_axis(1.0f, 0.0f, 0.0f, pitch, qp);
    M4 ry = quat_to_m4(qy), rp = quat_to_m4(qp);
    M4 rot = m4_mul(&ry, &rp);
    M4 trot = m4_mul(&tr, &rot);
    M4 view = m4_inverse(&trot);
    memcpy(out->viewMatrix, view.m, sizeof view.m);

    /* UpdateProjection: InfiniteZPerspective (blitML.h:261-278) */
    float f = 1.0f / tanf(fov / 2.0f);
    M4 proj;
    memset(&proj, 0, sizeof proj);
    proj.m[0] = f / (ww / wh);
    proj.m[5] = f;
    proj.m[11] = 1.0f;
    proj.m[14] = zNear;
    out->proj0 = proj.m[0];
    out->proj5 = proj.m[5];
    M4 pv = m4_mul(&proj, &view);
    memcpy(out->projectionViewMatrix, pv.m, sizeof pv.m);
    /* frustum planes: transpose(P).GetRow(r)[k] = P[k*4 + r]; NormalizePlane divides by |xyz| */
    float px[4], py[4];
    for (int k = 0; k < 4; ++k) {
        px[k] = proj.m[k * 4 + 3] + proj.m[k * 4 + 0];
        py[k] = proj.m[k * 4 + 3] + proj.m[k * 4 + 1];
    }
    float lx = sqrtf(px[0] * px[0] + px[1] * px[1] + px[2] * px[2]);
    float ly = sqrtf(py[0] * py[0] + py[1] * py[1] + py[2] * py[2]);
    out->frustumRight = px[0] / lx;
    out->frustumLeft = px[2] / lx;
    out->frustumTop = py[1] / ly;
    out->frustumBottom = py[2] / ly;
    out->lodTarget = (2.0f / out->proj5) * (1.0f / wh);
    out->pyramidWidth = pyrW;
    out->pyramidHeight = pyrH;
}
