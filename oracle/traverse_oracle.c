/*
 * TEST ORACLE — CPU restatement of libYafaRay's ray/primitive acceleration
 * semantics.  Test infrastructure only: tests/, __graft_entry__.smoke() and
 * bench.py's CPU-baseline leg call it as the checker; the product never links
 * it.  Parity of this restatement is pinned against the reference itself
 * (oracle/ref/kdtree_dump, built from the reference sources) through the
 * golden vectors in tests/golden/.
 *
 * What a kd-tree query returns does not depend on the tree's shape, only on
 * these reference rules, restated here operation by operation:
 *   - Möller–Trumbore triangle/quad test, same float operation order
 *     (include/geometry/shape/shape_polygon.h:126-176; vector dot/cross at
 *     include/geometry/vector.h:156-247);
 *   - primitive bounds and the tree bound grown by 0.1 % per axis, the offset
 *     computed in double and applied in float
 *     (src/accelerator/accelerator_kdtree_original.cc:89-103,
 *     include/geometry/primitive/primitive_face.h:139-153);
 *   - Smits slab crossing of that bound (include/geometry/bound.h:156-198);
 *   - dynamic ray bias t_min = max(ray.tmin, 0.1*min_raydist*|leave-enter|),
 *     shadow rays the bias alone (accelerator_kdtree_common.h:139,
 *     accelerator.h:64, 85);
 *   - acceptance 0 < t, t_min <= t < t_max (accelerator.h:122-145);
 *   - Accelerator::intersect / isShadowed ray set-up: t_max = FLT_MAX when
 *     tmax < 0, shadow origin advanced by tmin and t_max = tmax - 2*tmin
 *     (accelerator.h:89-111).
 * The reference resolves exact ties in t by traversal order; this oracle (and
 * the GPU path) take the lowest primitive index.  Ties only occur on shared
 * edges and are counted separately by the tests.
 *
 * Compiled with -ffp-contract=off so no multiply-add is fused: every
 * operation rounds like the reference's SSE code on x86-64.
 */
#include <float.h>
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define ORC_TRI_MARK 0xFFFFFFFFu
#define ORC_LEAF_MAX 4

typedef struct { float x, y, z; } v3;

static inline v3 vsub(v3 a, v3 b) { v3 r = {a.x - b.x, a.y - b.y, a.z - b.z}; return r; }
static inline float vdot(v3 a, v3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline v3 vcross(v3 a, v3 b)
{
	v3 r = {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
	return r;
}

/* shape_polygon.h:126-176.  Returns t (0 when no hit) and (u,v). */
static float mt_intersect(const v3 *vtx, int n, v3 from, v3 dir, float *uo, float *vo)
{
	const v3 edge_1 = vsub(vtx[1], vtx[0]);
	const v3 edge_2 = vsub(vtx[2], vtx[0]);
	const v3 pvec_2 = vcross(dir, edge_2);
	const float det_1_2 = vdot(edge_1, pvec_2);
	if(det_1_2 != 0.f)
	{
		const float inv_det_1_2 = 1.f / det_1_2;
		const v3 tvec = vsub(from, vtx[0]);
		float u = vdot(tvec, pvec_2) * inv_det_1_2;
		if(u >= 0.f && u <= 1.f)
		{
			const v3 qvec_1 = vcross(tvec, edge_1);
			const float v = vdot(dir, qvec_1) * inv_det_1_2;
			if(v >= 0.f && (u + v) <= 1.f)
			{
				const float t = vdot(edge_2, qvec_1) * inv_det_1_2;
				if(t > 0.f)
				{
					if(n == 3) { *uo = u; *vo = v; }
					else { *uo = u + v; *vo = v; }
					return t;
				}
			}
		}
		else if(n == 4)
		{
			const v3 edge_3 = vsub(vtx[3], vtx[0]);
			const v3 pvec_3 = vcross(dir, edge_3);
			const float det_2_3 = vdot(edge_2, pvec_3);
			if(det_2_3 != 0.f)
			{
				const float inv_det_2_3 = 1.f / det_2_3;
				u = vdot(tvec, pvec_3) * inv_det_2_3;
				if(u >= 0.f && u <= 1.f)
				{
					const v3 qvec_2 = vcross(tvec, edge_2);
					const float v = vdot(dir, qvec_2) * inv_det_2_3;
					if(v >= 0.f && (u + v) <= 1.f)
					{
						const float t = vdot(edge_3, qvec_2) * inv_det_2_3;
						if(t > 0.f) { *uo = u; *vo = u + v; return t; }
					}
				}
			}
		}
	}
	return 0.f;
}

typedef struct { float lo[3], hi[3]; } box;

typedef struct {
	box b;
	int32_t left;      /* internal: child index; leaf: -1 */
	int32_t right;     /* internal: child index; leaf: first slot in order[] */
	int32_t count;     /* leaf: number of primitives */
} node;

typedef struct orc_scene {
	uint32_t nf;
	v3 *vtx;           /* 4 per face (the 4th copies the 3rd for triangles) */
	uint8_t *nvtx;     /* 3 or 4 */
	box *pb;           /* primitive bounds */
	float bound[6];    /* reference tree bound (inflated) */
	node *nodes;
	uint32_t n_nodes;
	uint32_t *order;   /* leaf slots -> primitive index */
} orc_scene;

static void box_empty(box *b)
{
	for(int k = 0; k < 3; ++k) { b->lo[k] = FLT_MAX; b->hi[k] = -FLT_MAX; }
}
static void box_grow(box *b, const box *o)
{
	for(int k = 0; k < 3; ++k)
	{
		if(o->lo[k] < b->lo[k]) b->lo[k] = o->lo[k];
		if(o->hi[k] > b->hi[k]) b->hi[k] = o->hi[k];
	}
}
static float box_area(const box *b)
{
	const float dx = b->hi[0] - b->lo[0], dy = b->hi[1] - b->lo[1], dz = b->hi[2] - b->lo[2];
	if(dx < 0.f) return 0.f;
	return dx * dy + dy * dz + dz * dx;
}

/* ---- binned-SAH BVH of the oracle's own (shape irrelevant to results) ---- */
#define NBIN 16
static uint32_t build_rec(orc_scene *s, uint32_t *idx, uint32_t lo, uint32_t hi, const float *cen, uint32_t *next)
{
	const uint32_t me = (*next)++;
	node *nd = &s->nodes[me];
	box b; box_empty(&b);
	box cb; box_empty(&cb);
	for(uint32_t i = lo; i < hi; ++i)
	{
		box_grow(&b, &s->pb[idx[i]]);
		box c = {{cen[3 * idx[i]], cen[3 * idx[i] + 1], cen[3 * idx[i] + 2]},
		         {cen[3 * idx[i]], cen[3 * idx[i] + 1], cen[3 * idx[i] + 2]}};
		box_grow(&cb, &c);
	}
	nd->b = b;
	const uint32_t n = hi - lo;
	int axis = -1; float best = FLT_MAX; int best_bin = 0;
	if(n > ORC_LEAF_MAX)
	{
		for(int k = 0; k < 3; ++k)
		{
			const float ext = cb.hi[k] - cb.lo[k];
			if(!(ext > 0.f)) continue;
			box bb[NBIN]; uint32_t bc[NBIN];
			for(int j = 0; j < NBIN; ++j) { box_empty(&bb[j]); bc[j] = 0; }
			for(uint32_t i = lo; i < hi; ++i)
			{
				int j = (int)((cen[3 * idx[i] + k] - cb.lo[k]) / ext * NBIN);
				if(j >= NBIN) j = NBIN - 1;
				if(j < 0) j = 0;
				box_grow(&bb[j], &s->pb[idx[i]]); bc[j]++;
			}
			float ra[NBIN]; uint32_t rc[NBIN];
			box acc; box_empty(&acc); uint32_t c = 0;
			for(int j = NBIN - 1; j > 0; --j) { box_grow(&acc, &bb[j]); c += bc[j]; ra[j] = box_area(&acc); rc[j] = c; }
			box_empty(&acc); c = 0;
			for(int j = 0; j < NBIN - 1; ++j)
			{
				box_grow(&acc, &bb[j]); c += bc[j];
				if(c == 0 || rc[j + 1] == 0) continue;
				const float cost = box_area(&acc) * c + ra[j + 1] * rc[j + 1];
				if(cost < best) { best = cost; axis = k; best_bin = j; }
			}
		}
	}
	uint32_t mid = lo;
	if(axis >= 0)
	{
		const float ext = cb.hi[axis] - cb.lo[axis];
		uint32_t i = lo, j = hi;
		while(i < j)
		{
			int bj = (int)((cen[3 * idx[i] + axis] - cb.lo[axis]) / ext * NBIN);
			if(bj >= NBIN) bj = NBIN - 1;
			if(bj <= best_bin) ++i;
			else { --j; uint32_t t = idx[i]; idx[i] = idx[j]; idx[j] = t; }
		}
		mid = i;
	}
	if(axis < 0 && n > ORC_LEAF_MAX) mid = lo + n / 2; /* degenerate centroids: split by count */
	if(n <= ORC_LEAF_MAX || mid == lo || mid == hi)
	{
		if(n > ORC_LEAF_MAX) mid = lo + n / 2;
		else { nd->left = -1; nd->right = (int32_t)lo; nd->count = (int32_t)n; return me; }
	}
	const uint32_t l = build_rec(s, idx, lo, mid, cen, next);
	const uint32_t r = build_rec(s, idx, mid, hi, cen, next);
	nd = &s->nodes[me];
	nd->left = (int32_t)l; nd->right = (int32_t)r; nd->count = 0;
	return me;
}

orc_scene *orc_scene_create(const float *verts, uint32_t nv, const uint32_t *faces, uint32_t nf)
{
	(void)nv;
	orc_scene *s = (orc_scene *)calloc(1, sizeof(orc_scene));
	s->nf = nf;
	s->vtx = (v3 *)malloc(sizeof(v3) * 4 * (size_t)(nf ? nf : 1));
	s->nvtx = (uint8_t *)malloc((size_t)(nf ? nf : 1));
	s->pb = (box *)malloc(sizeof(box) * (size_t)(nf ? nf : 1));
	float *cen = (float *)malloc(sizeof(float) * 3 * (size_t)(nf ? nf : 1));
	box tb; box_empty(&tb);
	for(uint32_t i = 0; i < nf; ++i)
	{
		const int n = faces[4 * (size_t)i + 3] == ORC_TRI_MARK ? 3 : 4;
		s->nvtx[i] = (uint8_t)n;
		for(int k = 0; k < 4; ++k)
		{
			const uint32_t vi = faces[4 * (size_t)i + (k < n ? k : n - 1)];
			v3 p = {verts[3 * (size_t)vi], verts[3 * (size_t)vi + 1], verts[3 * (size_t)vi + 2]};
			s->vtx[4 * (size_t)i + k] = p;
		}
		/* primitive_face.h:139-153: min/max over the face's vertices */
		box b;
		for(int a = 0; a < 3; ++a)
		{
			const float *p0 = &s->vtx[4 * (size_t)i].x;
			b.lo[a] = p0[a]; b.hi[a] = p0[a];
			for(int k = 1; k < n; ++k)
			{
				const float c = (&s->vtx[4 * (size_t)i + k].x)[a];
				if(c < b.lo[a]) b.lo[a] = c;
				if(c > b.hi[a]) b.hi[a] = c;
			}
			cen[3 * (size_t)i + a] = 0.5f * (b.lo[a] + b.hi[a]);
		}
		s->pb[i] = b;
		/* Bound<float>{tree_bound_, all_bounds_[i]}: component-wise min/max */
		box_grow(&tb, &b);
	}
	if(nf == 0) { for(int a = 0; a < 3; ++a) { tb.lo[a] = 0.f; tb.hi[a] = 0.f; } }
	/* accelerator_kdtree_original.cc:99-103 */
	for(int a = 0; a < 3; ++a)
	{
		const double offset = (double)(tb.hi[a] - tb.lo[a]) * 0.001;
		tb.lo[a] -= (float)offset;
		tb.hi[a] += (float)offset;
		s->bound[a] = tb.lo[a];
		s->bound[3 + a] = tb.hi[a];
	}
	/* The oracle's own hierarchy tests boxes grown by 2^-18 of the coordinate
	 * plus 2^-18 of the scene extent, so float rounding in the box test never
	 * culls a primitive the Möller–Trumbore test would accept. */
	{
		float ext = 0.f;
		for(int a = 0; a < 3; ++a) if(tb.hi[a] - tb.lo[a] > ext) ext = tb.hi[a] - tb.lo[a];
		const float pad = ext * 3.81469727e-6f;
		for(uint32_t i = 0; i < nf; ++i)
			for(int a = 0; a < 3; ++a)
			{
				s->pb[i].lo[a] -= fabsf(s->pb[i].lo[a]) * 3.81469727e-6f + pad;
				s->pb[i].hi[a] += fabsf(s->pb[i].hi[a]) * 3.81469727e-6f + pad;
			}
	}
	s->order = (uint32_t *)malloc(sizeof(uint32_t) * (size_t)(nf ? nf : 1));
	for(uint32_t i = 0; i < nf; ++i) s->order[i] = i;
	s->nodes = (node *)malloc(sizeof(node) * 2 * (size_t)(nf ? nf : 1));
	uint32_t next = 0;
	if(nf) build_rec(s, s->order, 0, nf, cen, &next);
	s->n_nodes = next;
	free(cen);
	return s;
}

void orc_scene_destroy(orc_scene *s)
{
	if(!s) return;
	free(s->vtx); free(s->nvtx); free(s->pb); free(s->nodes); free(s->order); free(s);
}

void orc_scene_bound(const orc_scene *s, float *out6) { memcpy(out6, s->bound, sizeof(float) * 6); }

/* bound.h:156-198 (Smits).  Returns 1 and enter/leave when crossed. */
int orc_bound_cross(const float *bound6, const float *from, const float *dir, float t_max, float *enter, float *leave)
{
	const float *a = bound6, *g = bound6 + 3;
	const float p[3] = {from[0] - a[0], from[1] - a[1], from[2] - a[2]};
	float lmin = -FLT_MAX, lmax = FLT_MAX;
	for(int axis = 0; axis < 3; ++axis)
	{
		if(dir[axis] != 0.f)
		{
			const float inv_dir = 1.f / dir[axis];
			float ltmin, ltmax;
			if(inv_dir > 0.f) { ltmin = -p[axis] * inv_dir; ltmax = ((g[axis] - a[axis]) - p[axis]) * inv_dir; }
			else { ltmin = ((g[axis] - a[axis]) - p[axis]) * inv_dir; ltmax = -p[axis] * inv_dir; }
			if(axis == 0) { lmin = ltmin; lmax = ltmax; }
			else { lmin = ltmin > lmin ? ltmin : lmin; lmax = ltmax < lmax ? ltmax : lmax; }
			if((lmax < 0.f) || (lmin > t_max)) return 0;
		}
	}
	if((lmin <= lmax) && (lmax >= 0.f) && (lmin <= t_max)) { *enter = lmin; *leave = lmax; return 1; }
	return 0;
}

/* Conservative slab test of a (grown) box against [t0, t1]; *tn = entry. */
static inline int slab(const box *b, const float *o, const float *inv, float t0, float t1, float *tn)
{
	for(int k = 0; k < 3; ++k)
	{
		float n = (b->lo[k] - o[k]) * inv[k], f = (b->hi[k] - o[k]) * inv[k];
		if(n > f) { float t = n; n = f; f = t; }
		if(n != n) n = -FLT_MAX; /* 0*inf */
		if(f != f) f = FLT_MAX;
		if(n > t0) t0 = n;
		if(f < t1) t1 = f;
	}
	*tn = t0;
	return t0 <= t1 * 1.0000004f;
}

/* One query, mode 0 closest (Accelerator::intersect) or 1 shadow (isShadowed). */
static void query(const orc_scene *s, const float *r, int mode, int bruteforce, int32_t *prim, float *tout, float *uout, float *vout)
{
	float from[3] = {r[0], r[1], r[2]};
	const float dir[3] = {r[4], r[5], r[6]};
	const float tmin = r[3], tmax = r[7];
	float t_max;
	if(mode == 0) t_max = (tmax >= 0.f) ? tmax : FLT_MAX;
	else
	{
		for(int k = 0; k < 3; ++k) from[k] += dir[k] * tmin;   /* accelerator.h:106 */
		t_max = (tmax >= 0.f) ? tmax - 2 * tmin : FLT_MAX;     /* accelerator.h:108 */
	}
	*prim = -1; *tout = 0.f; *uout = 0.f; *vout = 0.f;
	float enter, leave;
	if(s->nf == 0 || !orc_bound_cross(s->bound, from, dir, t_max, &enter, &leave)) return;
	const float bias = 0.1f * 0.00005f * fabsf(leave - enter);
	const float t_min = (mode == 1) ? bias : (tmin > bias ? tmin : bias);
	const v3 F = {from[0], from[1], from[2]}, D = {dir[0], dir[1], dir[2]};
	float best = t_max; int32_t best_id = -1; float bu = 0.f, bv = 0.f;
	if(bruteforce)
	{
		for(uint32_t i = 0; i < s->nf; ++i)
		{
			float u, v;
			const float t = mt_intersect(&s->vtx[4 * (size_t)i], s->nvtx[i], F, D, &u, &v);
			if(t <= 0.f || t < t_min || t >= t_max) continue;
			if(mode == 1) { *prim = (int32_t)i; *tout = t; *uout = u; *vout = v; return; }
			if(t < best || (t == best && best_id >= 0 && (int32_t)i < best_id)) { best = t; best_id = (int32_t)i; bu = u; bv = v; }
		}
	}
	else
	{
		float inv[3];
		for(int k = 0; k < 3; ++k) inv[k] = 1.f / dir[k];
		uint32_t stack[128]; float stack_t[128]; int sp = 0;
		float tn_root;
		if(slab(&s->nodes[0].b, from, inv, 0.f, best, &tn_root)) { stack[sp] = 0; stack_t[sp] = tn_root; ++sp; }
		while(sp)
		{
			--sp;
			if(stack_t[sp] > best * 1.0000004f) continue;
			const node *nd = &s->nodes[stack[sp]];
			if(nd->left < 0)
			{
				for(int32_t j = 0; j < nd->count; ++j)
				{
					const uint32_t i = s->order[nd->right + j];
					float u, v;
					const float t = mt_intersect(&s->vtx[4 * (size_t)i], s->nvtx[i], F, D, &u, &v);
					if(t <= 0.f || t < t_min || t >= t_max) continue;
					if(mode == 1) { *prim = (int32_t)i; *tout = t; *uout = u; *vout = v; return; }
					if(t < best || (t == best && best_id >= 0 && (int32_t)i < best_id)) { best = t; best_id = (int32_t)i; bu = u; bv = v; }
				}
			}
			else
			{
				float ta, tb;
				const int ha = slab(&s->nodes[nd->left].b, from, inv, 0.f, best, &ta);
				const int hb = slab(&s->nodes[nd->right].b, from, inv, 0.f, best, &tb);
				if(ha && hb)
				{
					const int near_left = ta <= tb;
					stack[sp] = (uint32_t)(near_left ? nd->right : nd->left); stack_t[sp] = near_left ? tb : ta; ++sp;
					stack[sp] = (uint32_t)(near_left ? nd->left : nd->right); stack_t[sp] = near_left ? ta : tb; ++sp;
				}
				else if(ha) { stack[sp] = (uint32_t)nd->left; stack_t[sp] = ta; ++sp; }
				else if(hb) { stack[sp] = (uint32_t)nd->right; stack_t[sp] = tb; ++sp; }
			}
		}
	}
	if(best_id >= 0) { *prim = best_id; *tout = best; *uout = bu; *vout = bv; }
}

typedef struct {
	const orc_scene *s; const float *rays; uint32_t lo, hi; int mode, brute;
	int32_t *prim; float *t, *u, *v;
} job;

static void *worker(void *p)
{
	job *j = (job *)p;
	for(uint32_t i = j->lo; i < j->hi; ++i)
		query(j->s, j->rays + 8 * (size_t)i, j->mode, j->brute, j->prim + i, j->t + i, j->u + i, j->v + i);
	return NULL;
}

/* rays: 8 floats each (ox oy oz tmin dx dy dz tmax), the gbrt_ray layout.
 * threads <= 1: serial. */
void orc_trace(const orc_scene *s, const float *rays, uint32_t n, int mode, int bruteforce, int threads,
               int32_t *prim, float *t, float *u, float *v)
{
	if(threads < 1) threads = 1;
	if(threads > 256) threads = 256;
	pthread_t th[256]; job jobs[256]; int created[256];
	const uint32_t per = (n + (uint32_t)threads - 1) / (uint32_t)threads;
	int njobs = 0;
	for(int k = 0; k < threads; ++k)
	{
		uint32_t lo = (uint32_t)k * per, hi = lo + per;
		if(lo >= n) break;
		if(hi > n) hi = n;
		jobs[k] = (job){s, rays, lo, hi, mode, bruteforce, prim, t, u, v};
		created[k] = 0;
		if(threads > 1 && pthread_create(&th[k], NULL, worker, &jobs[k]) == 0) created[k] = 1;
		else worker(&jobs[k]);
		njobs = k + 1;
	}
	for(int k = 0; k < njobs; ++k)
		if(created[k]) pthread_join(th[k], NULL);
}

/* Exposed for unit tests of the triangle arithmetic. */
float orc_mt_intersect(const float *vtx12, int n, const float *from, const float *dir, float *u, float *v)
{
	v3 q[4];
	for(int k = 0; k < 4; ++k) { q[k].x = vtx12[3 * k]; q[k].y = vtx12[3 * k + 1]; q[k].z = vtx12[3 * k + 2]; }
	const v3 F = {from[0], from[1], from[2]}, D = {dir[0], dir[1], dir[2]};
	return mt_intersect(q, n, F, D, u, v);
}
