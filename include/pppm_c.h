/*
 * pppm_c.h - C ABI of the GB300 (sm_103a) implementation of tatsy-pppm's
 * probabilistic progressive photon mapping (PPM-APA) pass.
 *
 * The reference has no FFI: its interface is C++ methods taking
 * `const Scene&`, `const Camera&` and `const RenderParameters&`. Every entry
 * point below names the reference method it replaces (file:line within the
 * tatsy-pppm project). The C++ host mirror in tatsy-pppm_gb300/host/ keeps
 * the reference class names on top of these calls.
 *
 * Conventions
 *  - Every function returns an int status: PPPM_OK (0) or a negative
 *    PPPM_E_* code. Nothing aborts. pppm_last_error() describes the last
 *    failure of a context.
 *  - Array arguments may live in host memory or in device memory of the
 *    context's GPU (detected with CUDA unified addressing). Host arrays are
 *    staged through buffers owned by the context and are not retained after
 *    the call returns; a call that touches any host array synchronises its
 *    stream before returning. A call whose arrays are all on the device is
 *    enqueued on the context stream and returns without waiting
 *    (pppm_sync() waits and reports deferred kernel errors).
 *  - One context per host thread; the context owns all device memory it
 *    allocates. Calls on one context are not thread safe.
 *  - Triangles are 9 floats (p0, p1, p2); rays are 6 floats (origin,
 *    unit direction), vectors are xyz floats unless stated otherwise.
 */
#ifndef PPPM_C_H_
#define PPPM_C_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PPPM_OK 0
#define PPPM_E_ARG (-1)       /* invalid argument or size */
#define PPPM_E_CUDA (-2)      /* CUDA runtime error (message in pppm_last_error) */
#define PPPM_E_STATE (-3)     /* call out of order (no scene, no env, ...) */
#define PPPM_E_CAPACITY (-4)  /* an output or internal buffer was too small */
#define PPPM_E_UNDEFINED (-5) /* input whose reference behaviour is undefined */
#define PPPM_E_TIMEOUT (-6)   /* a bounded device-side loop ran out of iterations */

/* BSDF type bits (bsdf.h:19-26). */
#define PPPM_BSDF_LAMBERTIAN 0x01
#define PPPM_BSDF_SPECULAR 0x02
#define PPPM_BSDF_PHONG 0x04
#define PPPM_BSDF_REFRACTION 0x08
#define PPPM_BSDF_BSSRDF 0x10

/* Render modes. */
#define PPPM_MODE_COMPAT 0    /* the reference's semantics, quirks included */
#define PPPM_MODE_CANONICAL 1 /* textbook Knaus-Zwicker PPM-APA */
#define PPPM_MODE_CLASSIC 2   /* ProgressivePhotonMapping (classic PPM, progressive_photon_mapping.cc):
                                 per-pixel render points with their own radius and photon count,
                                 permuted Halton sampling, the reference's semantics */
#define PPPM_MODE_PATH_TRACING 3 /* PathTracing (path_tracing.cc:23-198), the reference's other integrator:
                                   one path per pixel per pass from the reference's row tapes (num_streams
                                   XorShift streams), env light at misses, max_bounce_eye = bounceLimit
                                   (64 in the reference); photons drive only the subsurface stage */

typedef struct pppm_ctx pppm_ctx;

/* One material (BSDF + optional dipole BSSRDF), replaces the factories
 * LambertianBRDF/SpecularBRDF/PhongBRDF/RefractionBSDF::factory
 * (brdf.cc:23-150) and DipoleBSSRDF::factory (bssrdf.cc:48-63). 56 bytes. */
typedef struct {
    int32_t type;       /* one PPPM_BSDF_* bit (not BSSRDF) */
    int32_t has_bssrdf; /* 1: BSDF::setBssrdf(DipoleBSSRDF(...)) (bsdf.cc:70-73) */
    float refl[3];      /* reflectance */
    float phong_n;      /* Phong exponent */
    float sigma_a[3];   /* dipole absorption */
    float sigmap_s[3];  /* dipole reduced scattering */
    float eta;          /* dipole relative IOR */
    float scale;        /* dipole distance scale */
} pppm_material;

/* Pinhole camera, replaces PerspectiveCamera (perspective_camera.cc:11-46).
 * fov is used as tan(fov*0.5) exactly like the reference (an angle in
 * radians; the reference's own driver passes 45.0). */
typedef struct {
    float eye[3];
    float dir[3];
    float up[3];
    float fov;
    int32_t width;
    int32_t height;
} pppm_camera;

/* Replaces RenderParameters (render_parameters.h:12) plus the constants of
 * ppm_probabilistic.cc (ALPHA, radius init, bounce limits, OMP streams). */
typedef struct {
    int32_t mode;           /* PPPM_MODE_* */
    int32_t num_streams;    /* RNG streams = OMP_NUM_CORE of the reference run (compat) */
    int64_t photons;        /* photons emitted per pass (RenderParameters::photons) */
    int32_t gather_photons; /* RenderParameters::gatherPhotons */
    int32_t max_bounce_photon; /* tracePhotons bounceLimit (64) */
    int32_t max_bounce_eye;    /* radiance bounceLimit (64) */
    uint32_t seed;          /* canonical-mode RNG seed */
    double gather_radius;   /* RenderParameters::gatherRadius */
    double alpha;           /* ALPHA (0.7) */
    double radius_scale;    /* r1 = radius_scale * |bbox diagonal| (0.1 in the reference) */
    float cell_factor;      /* hash-grid cell size: canonical = cell_factor * radius (>= 1) */
    int32_t flags;          /* PPPM_FLAG_* */
    uint32_t sss_time;      /* compat, scenes with a BSSRDF: the value time(NULL) returns when pass 1
                               seeds its subsurface photon streams (subsurface_integrator.cc:248);
                               pass t uses sss_time + t - 1 */
} pppm_params;

/* pppm_params.flags */
#define PPPM_FLAG_COUNT_TRAVERSAL 0x1 /* count BVH nodes visited / triangles tested */
#define PPPM_FLAG_LEARNED 0x2 /* canonical mode: learned photon proposal (MLP + vMF mixture, one-sample MIS
                                 with the reference's environment sampling, and optionally with the BSDF at
                                 Lambertian bounces, at a floor of 0.3; retrained every 2 passes); no
                                 reference counterpart */
#define PPPM_FLAG_LEARNED_FROZEN 0x4 /* with PPPM_FLAG_LEARNED: the same pipeline without training (the
                                        reference's sampling alone): the method without the network */
#define PPPM_FLAG_SAMPLER_QMC 0x8 /* compat mode: the RANDOM_SAMPLER_QUASI_MONTE_CARLO sampler type of
                                     ProgressivePhotonMappingProb::render (ppm_probabilistic.cc:58-73):
                                     stream i is Halton(200, true, i) (halton.cc) instead of XorShift(i) */

/* Per-pass statistics written by pppm_render_pass. */
typedef struct {
    int64_t photons_traced;  /* emitted photon paths (num_streams * ceil(P/N) in compat) */
    int64_t photons_stored;  /* photon records deposited (excluding phantoms) */
    int64_t phantom_photons; /* compat: default Photon() slots entering the map */
    int64_t photon_rays;     /* photon ray segments traced */
    int64_t eye_rays;        /* eye ray segments traced */
    int64_t gather_queries;  /* Lambertian hit points gathered */
    double radius;           /* global radius used in this pass */
    double ms_photon;        /* device time of the photon stage (ms) */
    double ms_grid;          /* hash-grid build (ms) */
    double ms_eye;           /* eye paths (ms) */
    double ms_gather;        /* gather (ms) */
    double ms_bounce;        /* photon bounce kernels only (ms) */
    int64_t kernel_launches; /* kernels launched by the pass */
    int64_t node_visits;     /* BVH nodes visited (PPPM_FLAG_COUNT_TRAVERSAL) */
    int64_t tri_tests;       /* triangles tested (PPPM_FLAG_COUNT_TRAVERSAL) */
    int64_t photon_node_visits; /* of which by photon rays */
    int64_t photon_tri_tests;
    int64_t gather_pairs;    /* canonical: photon-query pairs tested (PPPM_FLAG_COUNT_TRAVERSAL) */
    int64_t gather_inside;   /* canonical: pairs within the radius (PPPM_FLAG_COUNT_TRAVERSAL) */
    int64_t sss_points;      /* subsurface irradiance points (Poisson-disc samples) of this pass */
    int64_t sss_photons;     /* subsurface photons stored */
    double ms_subsurface;    /* subsurface stage before the photon pass (ms, includes host sampling) */
    double ms_subsurface_host; /* host time of the octree build loop (level syncs; overlaps the photon pass) (ms) */
    double ms_train;         /* learned proposal: training after this pass (ms) */
    double train_loss;       /* learned proposal: loss of the last training step */
    int64_t train_records;   /* learned proposal: records available to the last training */
} pppm_pass_stats;

/* ------------------------------------------------------------- lifetime */
/* device: CUDA ordinal. */
int pppm_create(int device, pppm_ctx** out);
int pppm_destroy(pppm_ctx* ctx);
const char* pppm_last_error(const pppm_ctx* ctx);
/* Waits for all work queued on the context stream. */
int pppm_sync(pppm_ctx* ctx);
/* The context's cudaStream_t, for callers that time or order work. */
void* pppm_stream(pppm_ctx* ctx);

/* ------------------------------------------------------------- scene */
/* Replaces Scene::add<T> (scene.h:38-50) + Scene::setAccelerator
 * (scene.cc:35-38) + QBVHAccel::construct (qbvh_accel.cc:139-203): uploads
 * the triangle soup (tri_xyz: 9*ntri floats, host), one material id per
 * triangle and builds the 4-wide BVH with the reference's topology. */
int pppm_scene_set(pppm_ctx* ctx, const float* tri_xyz, int64_t ntri, const int32_t* mat_id,
                   const pppm_material* mats, int32_t nmat);

/* Replaces Envmap::Envmap(file) (envmap.cc:28-36): rgb is w*h*3 floats of
 * the decoded equirect image (row 0 = top, as Image stores it); builds the
 * 64x64 importance pdf/cdf (envmap.cc:88-163) in double on the host.
 * The map stays with the context across pppm_scene_set; rgb = NULL with
 * w = h = 0 removes it (a Scene without setEnvmap: rays that leave the
 * scene see black, scene.cc:11-12). */
int pppm_env_set(pppm_ctx* ctx, const float* rgb, int32_t w, int32_t h);

/* Makes material mat_id (of the scene set last) emit radiance rgb (3
 * floats >= 0) from the front side of its triangles (the side of
 * (p1 - p0) x (p2 - p0)). No counterpart in the reference, whose only light
 * is the environment map. With emitters in the scene every photon leaves an
 * emitter: the emitter by area, a uniform point of it, a cosine direction
 * about its normal, flux Le * pi * (total emitter area) / photons; eye paths
 * add Le where they meet a front side. A scene with emitters needs no
 * environment map (eye rays that miss then see black) and renders in
 * canonical mode or with the path tracer (other modes: PPPM_E_ARG at
 * pppm_render_begin). pppm_scene_set clears all emission. */
int pppm_material_emission(pppm_ctx* ctx, int32_t mat_id, const float* rgb);

/* Envmap importance tables (envmap.cc:88-163), 4096 doubles each. */
int pppm_env_tables(pppm_ctx* ctx, double* pdf, double* cdf);

/* Rebuilds the environment's 64x64 cell tables with cell weight
 * luminance^exponent (0 <= exponent <= 8) in place of the reference's
 * luminance^2 (envmap.cc:128-153; exponent 2 restores the reference's tables
 * bit for bit). Photon fluxes follow the new pdf (area / (pdf * P)), so every
 * exponent renders the same expectation; exponent 1 is the plain non-learned
 * alternative to the reference's heuristic on skies with a small bright sun.
 * Applies to passes rendered after the call; pppm_env_set restores 2; not
 * part of a checkpoint. No counterpart in the reference (its exponent is
 * fixed). */
int pppm_env_importance(pppm_ctx* ctx, double exponent);

/* Replaces Envmap::sampleFromDir (envmap.cc:47-60): nearest-texel radiance
 * for n unit directions (3 floats each, any memory) into rgb (n x 3). */
int pppm_env_lookup(pppm_ctx* ctx, const float* dirs, int64_t n, float* rgb);

/* Replaces Envmap::samplePhoton (envmap.cc:62-86) + the cosine-hemisphere
 * draw of tracePhotons (ppm_probabilistic.cc:137-144) on explicit random
 * tapes: tapes is n x 5 doubles in draw order. pos: photon origin 50*dir_env,
 * dir: first ray direction, flux: photon flux (n x 3 floats each).
 * defined[i] = 0 where the draw lies past the last CDF entry, where the
 * reference reads outside its pdf table. */
int pppm_emit_photons(pppm_ctx* ctx, const double* tapes, int64_t n, int64_t num_photons, float* pos, float* dir,
                      float* flux, int32_t* defined);

/* Decodes a Radiance RGBE file image held in memory (the reference's
 * Image::loadHdr, image.cc:296-434) into w*h*3 floats. Call with rgb=NULL
 * to query the size. */
int pppm_hdr_decode(const uint8_t* bytes, int64_t nbytes, float* rgb, int64_t cap_floats, int32_t* w, int32_t* h);

/* Decodes a PLY file image held in memory as Trimesh::loadPly does
 * (trimesh.cc:139-217): the first line must be "ply", the format
 * binary_little_endian, the elements "vertex" and "face" only; the body is 3
 * little-endian floats per vertex (whatever properties the header declares)
 * and, per face, one uchar count and 3 int32 indices. Call with verts and
 * faces NULL to query nverts/nfaces. A header without end_header gives an
 * empty mesh (PPPM_OK, 0 and 0), as in the reference. Where the reference
 * aborts or exits (other formats or elements, zero counts, a polygon of more
 * than 3 vertices) and where it reads past the data or outside the vertex
 * array (truncated body, index out of range), this returns PPPM_E_ARG.
 * Blank header lines are skipped. */
int pppm_ply_decode(const uint8_t* bytes, int64_t nbytes, float* verts, int64_t vcap_floats, int32_t* faces,
                    int64_t fcap_ints, int64_t* nverts, int64_t* nfaces);

/* Placement of a mesh before Scene::add, on n double vertices (3 per
 * vertex) with the reference's arithmetic in its order:
 * Trimesh::translate (trimesh.cc:272-276), Trimesh::scale(sx, sy, sz)
 * (:278-288), Trimesh::putOnPlane(Plane(distance, normal)) (:290-300),
 * Trimesh::fitToBBox(BBox(bmin, bmax)) (:302-320). The scene holds FP32
 * triangles, so transformed vertices are rounded once when the scene is
 * set. */
int pppm_mesh_translate(double* v, int64_t n, const double move[3]);
int pppm_mesh_scale(double* v, int64_t n, double sx, double sy, double sz);
int pppm_mesh_put_on_plane(double* v, int64_t n, double distance, const double normal[3]);
int pppm_mesh_fit_bbox(double* v, int64_t n, const double bmin[3], const double bmax[3]);

/* ------------------------------------------------------------- stages */
/* Replaces QBVHAccel::intersect (qbvh_accel.cc:205-285) through
 * Scene::intersect (scene.cc:40-47): closest hit of n rays. tri: original
 * triangle id or -1; t: hit distance (1e20 on a miss); pos/nrm (optional,
 * may be NULL): hit position and geometric normal (3 floats each). The
 * traversal and triangle test reproduce the reference arithmetic, so ids
 * and t are bit-identical for the same float rays. */
int pppm_intersect(pppm_ctx* ctx, const float* rays, int64_t n, int32_t* tri, double* t, float* pos, float* nrm);

/* Replaces HashGrid<T>::operator[] bucket selection (hash_grid_detail.h:60-72):
 * bucket index of each point for a grid initialised with
 * init(hash_size, scale, bbox) (hash_grid_detail.h:26-31). bbmin: 3 doubles. */
int pppm_hash_points(pppm_ctx* ctx, const float* pts, int64_t n, int32_t hash_size, double scale,
                     const double* bbmin, uint32_t* out);

/* Replaces HashGrid<T>::init(hash_size, scale, bbox) + add(item i, boxmin[i],
 * boxmax[i]) for i = 0 .. n-1 (hash_grid_detail.h:26-52) and the bucket
 * vectors operator[] returns: boxes are n x 3 doubles each (host or device),
 * bbmin the 3 doubles of bbox.posMin(). Cell coordinates are
 * |(int)((v - bbmin) * scale)| per axis, so boxes reaching below bbmin fold
 * as in the reference. Output in CSR form: start (hash_size + 1 offsets) and
 * items (item ids), each bucket in the reference's insertion order (add
 * order; an item appears once per covered cell that hashes to the bucket).
 * *count = the number of entries; start and items NULL: count only; items
 * NULL: offsets only; cap < *count: PPPM_E_CAPACITY. At most 2^24 cells per
 * box (PPPM_E_CAPACITY) and fewer than 2^32 entries in all. */
int pppm_hashgrid_build(pppm_ctx* ctx, const double* boxmin, const double* boxmax, int64_t n, int32_t hash_size,
                        double scale, const double* bbmin, uint32_t* start, int32_t* items, int64_t cap,
                        int64_t* count);

/* Replaces PhotonMap::findKNN (photon_map.cc:24-26) -> KdTree::knnSearch
 * (kdtree_detail.h:90-132) with the reference's argument order
 * (numTargetPhotons lands in epsilon, targetRadius in k). Results per query
 * in the reference's order (farthest first): idx (m x cap), cnt (m). */
int pppm_knn(pppm_ctx* ctx, const float* photon_pos, int64_t n, const float* queries, int64_t m,
             int32_t num_target_photons, double target_radius, int32_t* idx, int32_t* cnt, int32_t cap);

/* Replaces KdTree<T>::knnSearch(point, KnnQuery(type, epsilon, k), results)
 * (kdtree.h:13-24, kdtree_detail.h:88-132) over n points (3 floats each):
 * type is PPPM_KNN_EPSILON_BALL and/or PPPM_KNN_K_NEAREST as KnnSearchType;
 * without EPSILON_BALL the ball is unbounded. K_NEAREST: the k nearest
 * points strictly within epsilon (k <= 64 and <= cap); EPSILON_BALL alone:
 * every point within epsilon, refused with PPPM_E_CAPACITY when a query has
 * min(cap, 64) or more. Results per query farthest first (the max-heap's pop
 * order): idx (m x cap point indices), cnt (m). k < 1 with K_NEAREST returns
 * PPPM_E_UNDEFINED (the reference reads an empty queue). */
#define PPPM_KNN_EPSILON_BALL 0x01
#define PPPM_KNN_K_NEAREST 0x02
int pppm_kdtree_knn(pppm_ctx* ctx, const float* points, int64_t n, const float* queries, int64_t m, int32_t type,
                    double epsilon, int32_t k, int32_t* idx, int32_t* cnt, int32_t cap);

/* Replaces the Lambertian gather of ProgressivePhotonMappingProb::radiance
 * (ppm_probabilistic.cc:300-335). photons: n records of 8 floats
 * (pos xyz, flux xyz, normal packed as float bits of an int, unused);
 * queries: m records of 12 floats (pos xyz, normal xyz, refl xyz,
 * weight xyz = path throughput / roulette). mode COMPAT reproduces the
 * reference (kNN with k=(int)radius, eps=gather_photons, cone filter);
 * CANONICAL sums refl*flux/pi over photons within `radius` whose normal
 * faces the query normal, divided by pi*radius^2. out: m x 3 radiance
 * (weight included). phantoms: number of default Photon() records at the
 * origin that the compat map contains (ppm_probabilistic.cc:202-207). */
int pppm_gather(pppm_ctx* ctx, int32_t mode, const float* photons, int64_t n, int64_t phantoms,
                const float* queries, int64_t m, double radius, int32_t gather_photons, float* out);

/* Replaces DipoleBSSRDF::operator() (bssrdf.cc:92-104): Rd(d^2) per colour
 * channel for the dipole parameters of `mat` (sigma_a, sigmap_s, eta,
 * scale), including the reference's fast_exp approximation
 * (vector3d.cc:11-16). d2: n floats, rgb: n x 3. */
int pppm_dipole_rd(pppm_ctx* ctx, const pppm_material* mat, const float* d2, int64_t n, float* rgb);

/* Device self-check of the dipole's fast_exp (vector3d.cc:11-16): the
 * render evaluates it in 64-bit integer arithmetic for |y| <= 700 (FP64 runs
 * at a small fraction of the FP32 rate on this GPU) and in double outside.
 * Over the float bit patterns [begin, end) (end <= 2^32) counts the
 * arguments the integer form covers and, of those, the ones whose result
 * differs in any bit from the double form. */
int pppm_fast_exp_check(pppm_ctx* ctx, uint64_t begin, uint64_t end, uint64_t* covered, uint64_t* differ);

/* Replaces SubsurfaceIntegrator::irradiance (subsurface_integrator.cc:234-238)
 * over an octree built like Octree::construct (subsurface_integrator.cc:67-145)
 * from n irradiance points of 10 floats (pos xyz, normal xyz, area,
 * irradiance rgb): (1/pi)(1 - Fdr) * sum of Rd(d^2) * E * A over the nodes
 * accepted with threshold max_error. queries: m x 3, rgb: m x 3. Repeated
 * points return PPPM_E_UNDEFINED (the reference's recursion never ends). */
int pppm_dipole_irradiance(pppm_ctx* ctx, const pppm_material* mat, const float* ipts, int64_t n, double max_error,
                           const float* queries, int64_t m, float* rgb);

/* Replaces sampler::poissonDisk (sampler.cc:36-101): dart throwing over the
 * triangle soup (9 floats each, host) with minimum distance min_dist, on the
 * GPU with the reference's exact result. The candidate draws come from the
 * XorShift state rng_state (4 words, advanced in place; the reference uses a
 * process-wide XorShift seeded 0, whose initial state is XorShift(0)); the
 * acceptance order follows the reference's RandomQueue seeded -1 and its
 * hash grid. Writes up to cap points and triangle normals (3 floats each,
 * host) and the total count. */
int pppm_poisson_disk(pppm_ctx* ctx, const float* tri_xyz, int64_t ntri, double min_dist, uint32_t* rng_state,
                      float* pts, float* nrm, int64_t cap, int64_t* count);

/* Replaces SubsurfaceIntegrator::buildPhotonMap (subsurface_integrator.cc:
 * 240-327) as SubsurfaceIntegrator::initialize calls it: params->photons
 * env-map photons from num_streams streams, seeded XorShift(sss_time + t - 1
 * + i) in compat mode, up to 64 bounces, a record at every BSSRDF hit with
 * roulette on the mean flux. out: the records (n x 8 floats: position,
 * flux, packed normal, path index bits), *n their count (out NULL or cap
 * too small: count only). Sets up the context for this stage alone: any
 * active render of the context ends. The scene needs a BSSRDF material
 * (else PPPM_E_STATE). */
int pppm_subsurface_photons(pppm_ctx* ctx, const pppm_params* params, int32_t t, float* out, int64_t cap, int64_t* n);

/* Replaces SubsurfaceIntegrator::irradianceWithPM (subsurface_integrator.cc:
 * 329-365) over an injected photon map: photons are n records of 8 floats
 * (pos xyz, flux xyz, 2 unused), points m records of 6 floats (pos xyz,
 * normal xyz). As in the reference, findKNN receives (num_photons,
 * gather_radius), so k = (int)gather_radius nearest photons within distance
 * num_photons; the normal filter is |n.(p-q)|/|p-q| < gather_photons^2 *
 * 0.01; the cone-filtered flux weights the unfiltered list's photon i with
 * the i-th kept distance. out: m x 3 irradiance. */
int pppm_subsurface_photon_irradiance(pppm_ctx* ctx, const float* photons, int64_t n, const float* points, int64_t m,
                                      int64_t num_photons, double gather_radius, int32_t gather_photons, float* out);

/* Forward pass of the learned photon proposal network (no counterpart in
 * the reference): params is the flat FP32 parameter vector (W1[64][80] b1[64]
 * W2[64][64] b2 W3[64][64] b3 W4[40][64] b4[40], PPPM_MLP_PARAMS floats),
 * pos/nrm n x 3 floats, bbox 6 doubles (min xyz, max xyz) normalising the
 * positions of the input encoding. out: n x 40 raw outputs (8 lobes x weight
 * logit, mean xyz, log kappa). FP16 tensor-core GEMMs, FP32 accumulation. */
#define PPPM_MLP_PARAMS 16104
int pppm_mlp_forward(pppm_ctx* ctx, const float* params, const float* pos, const float* nrm, int64_t n,
                     const double* bbox, float* out);

/* Settings of the learned proposal for the next pppm_render_begin with
 * PPPM_FLAG_LEARNED (no counterpart in the reference). retrain_every: passes
 * between trainings (2); steps: Adam steps per training (2); batch: records
 * per step (65536); lr: Adam learning rate (4e-3); floor_bsdf: probability of
 * the reference's own sampling (environment cell draw, BSDF lobe) in the
 * one-sample MIS mixtures (0.3); max_log_kappa: upper
 * clamp of the lobes' log concentration (7); guide_bounces: 1 to guide
 * Lambertian bounces as well as the environment direction of emission, 0 for
 * emission only (0). Values < 0 (guide_bounces) or <= 0 (the others) keep the
 * current setting. */
int pppm_learned_config(pppm_ctx* ctx, int32_t retrain_every, int32_t steps, int64_t batch, float lr,
                        float floor_bsdf, float max_log_kappa, int32_t guide_bounces);

/* Loss and gradient of the proposal network on n training records (10
 * floats each: pos xyz, normal xyz, unit direction xyz, weight w >= 0): the
 * weighted negative log-likelihood  -sum_i w_i log q(d_i | x_i) / sum_i w_i
 * of the directions under the vMF mixture, back-propagated with FP16 tensor-
 * core GEMMs and FP32 accumulation. grad: PPPM_MLP_PARAMS floats (same
 * layout as params); loss: one float. No counterpart in the reference. */
int pppm_mlp_grad(pppm_ctx* ctx, const float* params, const float* records, int64_t n, const double* bbox,
                  float* grad, float* loss);

/* Halton(200, true, seed)::request (halton.cc:88-152) values of requests
 * 0 .. count-1 (n <= 200 numbers each) into out (count x n doubles), the
 * sampler of classic PPM, evaluated on the GPU in the reference's order. */
int pppm_halton(pppm_ctx* ctx, uint32_t seed, int32_t count, int32_t n, double* out);

/* Allocation-free variant of pppm_knn (same arguments and results) for
 * callers that cannot let a library allocate GPU memory: programs that own
 * all device memory under a fixed budget, frame loops that must not stall on
 * cudaMalloc, or code that must not create a pppm context. It needs no
 * context and calls no cudaMalloc/cudaFree or allocating library routine.
 * Every array must already be device memory of the current device (or
 * managed memory); host memory and another GPU's memory return PPPM_E_ARG.
 * Work runs on `stream` (a cudaStream_t, NULL = the default stream) and the
 * call waits for it before returning. Scratch lives in one fixed device
 * array of about 6.6 MB that every GPU loading the library holds until exit;
 * n above PPPM_NOALLOC_MAX_PHOTONS returns PPPM_E_CAPACITY. The first call
 * on a device looks up that array's address (issue it before any stream
 * capture); resetting that device (cudaDeviceReset) afterwards is not
 * supported. Calls share the array, so calls that overlap on the GPU race.
 * No counterpart in the reference. */
#define PPPM_NOALLOC_MAX_PHOTONS (1 << 17)
int pppm_knn_noalloc(const float* photon_pos, int64_t n, const float* queries, int64_t m, int32_t num_target_photons,
                     double target_radius, int32_t* idx, int32_t* cnt, int32_t cap, void* stream);

/* ------------------------------------------------------------- render */
/* Replaces the set-up half of ProgressivePhotonMappingProb::render
 * (ppm_probabilistic.cc:24-79): radius init, RNG streams, zeroed buffer. */
int pppm_render_begin(pppm_ctx* ctx, const pppm_camera* cam, const pppm_params* params);

/* One pass t (1-based) of the render loop (ppm_probabilistic.cc:80-96):
 * tracePhotons, photon map build, traceRays + gather, radius update. */
int pppm_render_pass(pppm_ctx* ctx, int32_t t, pppm_pass_stats* stats);

/* The next `count` passes of a canonical render as one CUDA graph launch (no
 * counterpart in the reference, whose render() loops over passes on the
 * host). Only for canonical renders without subsurface scattering, learned
 * proposal or traversal counting (else PPPM_E_STATE). The photon buffer, the
 * grid table and the sort buffers are sized before the capture for 1.5x the
 * most photons one earlier pass stored (a render with no pass done runs pass
 * 1 normally first); a captured pass that stores more returns
 * PPPM_E_CAPACITY after the launch, with the render left invalid. Results
 * equal those of pppm_render_pass up to the order of float sums. stats:
 * count entries (or NULL); for captured passes ms_photon (emission and
 * bounces, the eye paths beside them), ms_bounce and ms_gather (grid build
 * and gather) are device times, ms_grid and ms_eye 0. */
int pppm_render_graph(pppm_ctx* ctx, int32_t count, pppm_pass_stats* stats);

/* Advances an active render by `count` passes without rendering them: the
 * pass count, the radius schedule and (compat, path tracing) the streams'
 * tapes move on as if the passes had run, and nothing is accumulated (no
 * counterpart in the reference). For sharding the passes of one image over
 * processes or GPUs: a process that renders passes t = r + 1, r + 1 + n, ...
 * (skipping the others) accumulates exactly those passes, and the sum of
 * the n accumulators is the render of all passes up to the order of float
 * sums. Not for classic PPM, the subsurface stage or the learned proposal
 * (their passes depend on earlier ones): PPPM_E_STATE. */
int pppm_render_skip(pppm_ctx* ctx, int32_t count);

/* Launch-shape knobs of an active render, applied from the next pass on
 * (values <= 0 keep the current one): hash-grid cell factor (>= 1), photon
 * bounce and eye kernel blocks per SM (grid caps; bounce: default 64, at
 * most 64; eye: default 128, at most 128).
 * None changes results beyond the order
 * of floating-point accumulation; the batch autotuner sets them. No
 * counterpart in the reference. */
int pppm_render_tune(pppm_ctx* ctx, float cell_factor, int32_t bounce_blocks_per_sm, int32_t eye_blocks_per_sm);

/* Every launch-shape knob of a render. No field changes what a pass
 * computes (the same photon paths, deposits, eye paths and gather sets):
 * each only moves work between launches, lanes or tiles, and so may change
 * the order in which deposits are appended and the gather sums them. */
typedef struct pppm_tune {
    float cell_factor;             /* hash-grid cell edge / radius, >= 1 */
    int32_t bounce_blocks_per_sm;  /* photon kernel grid cap, 1..64 */
    int32_t eye_blocks_per_sm;     /* eye kernel grid cap, 1..128 */
    int32_t refill;                /* persistent photon kernel: lanes of a warp with their closest hit
                                      before the warp shades them and takes new paths, 1..32 */
    int32_t exact_batch;           /* lanes waiting for double-precision triangle tests before a
                                      warp runs them together, 1..32 */
    int32_t gather_stage;          /* canonical gather: photons per warp tile, a multiple of 32 in
                                      32..256 */
    int32_t query_sub_bits;        /* canonical gather: query sort key with 2^bits sub-cells per
                                      axis, 0..3 */
} pppm_tune;

/* Sets the knobs of an active render from the next pass on; a field < 0
 * (cell_factor <= 0) keeps its current value, a value out of range is
 * PPPM_E_ARG and changes nothing. render_begin restores the defaults
 * (1, 64, 128, 24, 12, 128, and 3 query sub-cell bits where the query sort
 * keeps 4096 cell buckets with them, 1080p and up; fewer for smaller
 * images, at least 1). No counterpart in the reference. */
int pppm_render_tune_ex(pppm_ctx* ctx, const pppm_tune* tune);

/* The knobs the next pass of the active render will use. */
int pppm_render_get_tune(pppm_ctx* ctx, pppm_tune* out);

/* The linear accumulation buffer after the last pass (not divided by the
 * pass count, not flipped): w*h*3 floats, row y = camera pixel row y. */
int pppm_render_read(pppm_ctx* ctx, float* accum);

/* The image the reference writes after a pass (ppm_probabilistic.cc:96-106):
 * accumulation / t with rows flipped (result(x, H - 1 - y) = buffer(x, y) / t),
 * Image::gamma(2.2, true) (image.cc:202-212), then Image::toByte
 * (image.cc:530-533). tonemap = 1 applies Image::tonemap first (image.cc:
 * 498-524: Reinhard, a = 0.18, log-average and maximum luminance of the
 * image). The arithmetic is the reference's, in double, on the FP32
 * accumulator. rgb8: w*h*3 bytes, host or device. */
int pppm_render_image(pppm_ctx* ctx, int32_t tonemap, uint8_t* rgb8);

/* The same output stage on an explicit accumulation buffer (w*h*3 floats,
 * host or device, row y = camera row y, the sum of `passes` passes): the
 * lines of ppm_probabilistic.cc:96-106 that fill _result and call
 * Image::gamma(2.2, true), with Image::tonemap (image.cc:498-524) first
 * when tonemap = 1, and Image::toByte (image.cc:530-533) as Image::savePng
 * applies it. rgb8: w*h*3 bytes, host or device. */
int pppm_image_bytes(pppm_ctx* ctx, const float* accum, int32_t w, int32_t h, int32_t passes, int32_t tonemap,
                     uint8_t* rgb8);

/* PNG file (8-bit RGB, no interlace) of w*h*3 bytes (host), in place of
 * stbi_write_png in Image::savePng (image.cc:484-495). The zlib stream holds
 * stored deflate blocks, one per row, so the file is larger than stb's but
 * decodes to the same pixels. out = NULL: *size only; else out must hold
 * *size bytes (PPPM_E_CAPACITY). Host only: needs no context and no GPU. */
int pppm_png_encode(const uint8_t* rgb8, int32_t w, int32_t h, uint8_t* out, int64_t cap, int64_t* size);

/* Checkpoint of the current render (no counterpart in the reference): the
 * camera, parameters, pass count, radius, tuned launch shapes, accumulation
 * buffer, per-stream XorShift states, the Poisson sampler's XorShift state,
 * classic PPM's render points and the learned proposal's network, Adam
 * moments, importance grids and pending records. out = NULL: *size only.
 * The learned proposal's settings (pppm_learned_config) are not part of it. */
int pppm_render_save(pppm_ctx* ctx, uint8_t* out, int64_t cap, int64_t* size);
/* Resumes a render from a checkpoint into a context that holds the same
 * scene and environment map (else PPPM_E_STATE): the next pppm_render_pass
 * continues with the saved pass count + 1. */
int pppm_render_load(pppm_ctx* ctx, const uint8_t* in, int64_t size);

/* ProgressivePhotonMappingProb::render (ppm_probabilistic.cc:24-121) minus
 * the PNG side effects: begin + `passes` passes + read. */
int pppm_render(pppm_ctx* ctx, const pppm_camera* cam, const pppm_params* params, int32_t passes, float* accum);

/* Photon records of the last pass: n x 8 floats (pos xyz, flux xyz, packed
 * normal, emitted path index as float bits of an int; in compat mode the
 * reference's thread of the path is index / ceil(P/N)). The records of one
 * path appear in bounce order. Returns the count in *n. */
int pppm_render_photons(pppm_ctx* ctx, float* out, int64_t cap, int64_t* n);

/* Gather queries (Lambertian hit points of the eye paths) of the last
 * PPM-APA pass, the hit points that radiance() (ppm_probabilistic.cc:300-335)
 * gathers at: n x 12 floats (position xyz, pixel index; oriented normal
 * xyz, specular and refractive bounces before the hit; path weight *
 * reflectance / roulette xyz, hit triangle id; the pixel index, bounces and
 * triangle id as float bits of an int), in the order the eye kernel wrote
 * them. Returns the count in *n. For parity checks of single hit points; no
 * counterpart in the reference. */
int pppm_render_queries(pppm_ctx* ctx, float* out, int64_t cap, int64_t* n);

/* ------------------------------------------------------------- batch */
/* Many uneven render jobs (each with its own scene, env map, camera and
 * parameters) run together on one GPU. No counterpart in the reference. */
typedef struct pppm_batch pppm_batch;

typedef struct {
    const float* tri_xyz;     /* 9 * ntri floats (host) */
    int64_t ntri;
    const int32_t* mat_id;    /* ntri */
    const pppm_material* mats;
    int32_t nmat;
    const float* env_rgb;     /* env_w * env_h * 3 floats (host) */
    int32_t env_w, env_h;
    pppm_camera camera;
    pppm_params params;
    int32_t passes;
} pppm_job;

typedef struct {
    int32_t passes;
    int32_t bounce_blocks_per_sm; /* launch shape chosen by the autotuner */
    int32_t eye_blocks_per_sm;
    float cell_factor;
    int64_t rays;                 /* photon + eye ray segments traced */
    double ms_total;              /* wall time of the job's passes */
    double ms_pass_p50, ms_pass_p99;
    double batch_wall_ms;         /* wall time of the whole pppm_batch_run */
    int32_t graph_passes;         /* passes of this job run inside the batch graph */
    double batch_graph_ms;        /* capture, instantiation and run of the batch graph */
    double batch_graph_capture_ms;     /* of which recording the passes */
    double batch_graph_instantiate_ms; /* of which cudaGraphInstantiate */
    int32_t refill;               /* the other knobs chosen (pppm_tune) */
    int32_t exact_batch;
    int32_t gather_stage;
    int32_t query_sub_bits;
    int32_t tune_passes;          /* passes spent on tuning (real passes of the render) */
    int32_t tune_candidate;       /* index of the candidate kept, -1 without tuning */
} pppm_job_stats;

int pppm_batch_create(int device, pppm_batch** out);
int pppm_batch_destroy(pppm_batch* batch);
const char* pppm_batch_last_error(const pppm_batch* batch);
/* Copies nothing it does not need: the scene and env map are uploaded and
 * the BVH built here. */
int pppm_batch_submit(pppm_batch* batch, const pppm_job* job, int32_t* job_id);
/* use_graph = 1 (the default): pppm_batch_run records the passes after the
 * first of every canonical job without subsurface scattering or learned
 * proposal into two CUDA graphs, each launched once: the tuning passes of
 * all jobs, then the remaining passes with each job's chosen knobs (one
 * branch per job, the branches chained into graph_lanes lanes; 0 = 2 x
 * max_concurrent); 0 runs every pass through pppm_render_pass. */
int pppm_batch_config(pppm_batch* batch, int32_t use_graph, int32_t graph_lanes);
/* Runs every job's passes: up to max_concurrent jobs at once (one host
 * worker and one stream each, longest first), then the batch graphs (see
 * pppm_batch_config). autotune = 1: a job of P passes tries up to
 * min(6, (P - 2) / 3) candidate settings of every pppm_tune knob, three
 * interleaved passes each, and renders its remaining passes with the one of
 * lowest median device time per pass (jobs under 8 passes are not tuned). */
int pppm_batch_run(pppm_batch* batch, int32_t autotune, int32_t max_concurrent);
/* A job's accumulation buffer (as pppm_render_read) and statistics. */
int pppm_batch_result(pppm_batch* batch, int32_t job_id, float* accum, pppm_job_stats* stats);

#ifdef __cplusplus
}
#endif

#endif /* PPPM_C_H_ */
