/* pfem_remesh.h - the host remesh between device steps, in C++ (libpfemremesh.so).
 *
 * Replaces Mesh::remesh (srcs/mesh/Mesh.cpp:919-926):
 *   laplacianSmoothingBoundaries (Mesh.cpp:580-760) -> addNodes (:27-147) -> removeNodes
 *   (:928-1017) -> checkBoundingBox (:149-207) -> triangulateAlphaShape (Mesh2D.cpp:32-251,
 *   Mesh3D.cpp:36-286, with deleteFlyingNodes, Mesh.cpp:251-331)
 * with the Delaunay triangulation computed here (incremental insertion with exact predicates)
 * where the reference calls CGAL.  The result is what pfg_upload_mesh_remap takes: positions,
 * flags, connectivity, facets, and per new node the old nodes its states come from.
 *
 * Arrays follow include/pfem_gpu.h: positions field-major (dim x n), connectivity (dim+1) x
 * n_elems, facets dim x n_facets, flags one byte per node (PFG_NODE_* bits).
 *
 * Errors: every call returns 0 on success, a negative code otherwise; pfr_last_error() gives
 * the message of the calling thread's last failure.  Calls are thread-safe on distinct meshes.
 */
#ifndef PFEM_REMESH_H
#define PFEM_REMESH_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define PFR_API __attribute__((visibility("default")))
#else
#define PFR_API
#endif

#define PFR_OK 0
#define PFR_ERR_INVALID -1   /* bad argument                                            */
#define PFR_ERR_NOMEM -2     /* host allocation failed                                  */
#define PFR_ERR_INTERNAL -3  /* triangulation failed (point location left the hull)     */

/* The Mesh block of a problem file (damBreakKoshizukaIncomp.lua:6-17). */
typedef struct pfr_params {
    int32_t dim;                            /* 2 or 3                                        */
    int32_t add_on_fs;                      /* addOnFS                                       */
    int32_t delete_flying_nodes;            /* deleteFlyingNodes                             */
    int32_t laplacian_smoothing_boundaries; /* laplacianSmoothingBoundaries                  */
    double hchar;                           /* hchar                                         */
    double alpha;                           /* alpha (alpha shape radius alpha * hchar)      */
    double omega;                           /* omega (addNodes: element size > omega h^d)    */
    double gamma;                           /* gamma (removeNodes: distance < gamma h)       */
    double jitter;                          /* the triangulation sees every node moved by
                                               U(-jitter, jitter) * hchar per coordinate (a
                                               counter-based hash of its index), which breaks
                                               the co-spherical ties of wall lattices as CGAL's
                                               symbolic perturbation does; all geometry uses
                                               the true positions.  Default 1e-6 in 3D, 0 in 2D */
    int32_t has_bounding_box;               /* boundingBox given                             */
    int32_t single_triangulation;           /* 0: 3D clouds of 16384 nodes or more with a
                                               perturbation are triangulated in cells on up to
                                               16 threads (the same simplices; the element order
                                               depends only on the node count); 1: always one
                                               triangulation                                  */
    double bounding_box[6];                 /* xmin, ymin(, zmin), xmax, ymax(, zmax)        */
} pfr_params;

typedef struct pfr_mesh pfr_mesh;

/* Defaults of the reference's dam-break problem files for `dim` and `hchar`:
 * alpha 1.2, omega 0.7, gamma 0.2, addOnFS false, deleteFlyingNodes true,
 * laplacianSmoothingBoundaries true, no bounding box. */
PFR_API int pfr_default_params(int32_t dim, double hchar, pfr_params* p);

/* One Mesh::remesh of the mesh (pos, flags, conn) whose positions the step already moved.
 * flags carry the free-surface bits of the last triangulation.  On success *out holds the new
 * mesh and, per new node, up to dim+1 old nodes whose states it takes (their mean). */
PFR_API int pfr_remesh(const pfr_params* p, int32_t n_nodes, const double* pos, const uint8_t* flags,
                       int32_t n_elems, const int32_t* conn, pfr_mesh** out);

/* Mesh::triangulateAlphaShape of a node cloud alone (the initial mesh of a problem): the
 * alpha shape of the Delaunay triangulation, free-surface flags, flying nodes removed when
 * p->delete_flying_nodes.  The origin table names the input node of each output node. */
PFR_API int pfr_alpha_shape(const pfr_params* p, int32_t n_nodes, const double* pos, const uint8_t* flags,
                            pfr_mesh** out);

/* Sizes of a result. */
PFR_API int pfr_mesh_counts(const pfr_mesh* m, int32_t* n_nodes, int32_t* n_elems, int32_t* n_facets);

/* Copy a result out.  Any pointer may be null.  origin is n_nodes x (dim+1), row-major,
 * padded with -1 (one source for a node that survived, dim+1 for a node added at a centroid). */
PFR_API int pfr_mesh_read(const pfr_mesh* m, double* pos, uint8_t* flags, int32_t* conn, int32_t* facets,
                          int32_t* facet_elm, int32_t* facet_out, int32_t* origin);

PFR_API void pfr_mesh_free(pfr_mesh* m);

/* Message of this thread's last failed call. */
PFR_API const char* pfr_last_error(void);

#ifdef __cplusplus
}
#endif

#endif /* PFEM_REMESH_H */
