/*
 * nekmesh.h -- host-side mesh ingestion for the solve path: the reference's
 * mesh (.re2) and connectivity (.co2) files, vertex connectivity computed
 * from element corners, the global numbering of GLL points and the GLL
 * coordinates of straight-sided elements.  These produce the arrays
 * nekgpu_setup takes (glo_num, and the coordinates the geometric factors are
 * computed from) for meshes that are not boxes.
 *
 * Host code only: no GPU is touched.  Arrays are the reference's layouts:
 * element corners (2^ndim per element) in the file's (preprocessor) corner
 * order unless a name says "tensor" order (corner i + 2 j + 4 k); faces in
 * the preprocessor face order the reference keeps cbc/bc in.  Element and
 * vertex numbers are 1-based, as in the reference.
 *
 * Status: 0 or a negative NEKGPU_E* code (nekgpu.h); NEKGPU_EIO for a file
 * that cannot be read or does not follow the format.  nekmesh_last_error()
 * gives the message of the calling thread's last failure.
 */
#ifndef NEKMESH_H
#define NEKMESH_H
#include <stdint.h>

#include "nekgpu.h"

#ifdef __cplusplus
extern "C" {
#endif

#define NEKGPU_EIO (-8) /* file missing, short or not in the expected format */

int nekmesh_last_error(char *buf, const int *buflen);

/* ---- .re2 (core/reader_re2.f) -------------------------------------------- */
/* Reads a whole .re2 file: the 80-byte header (read_re2_hdr :543-620,
 * versions #v001 with 4-byte words, #v002/#v003/#v004 with 8-byte words),
 * the byte-order test value 6.54321, the element records (group and corner
 * coordinates, readp_re2_mesh :68-157, buf_to_xyz :430-471), the curved-side
 * records (readp_re2_curve :159-286, buf_to_curve :473-501) and every
 * boundary-condition section present (readp_re2_bc :288-428, buf_to_bc
 * :503-541).  Files of either byte order are read. */
int nekmesh_re2_open(const char *path, int64_t *mesh);
/* nelgt, ndim, nelgv from the header; wdsize 4 or 8; the number of
 * curved-side records; the number of boundary-condition sections. */
int nekmesh_re2_header(const int64_t *mesh, int *nelgt, int *ndim, int *nelgv, int *wdsize,
                       int64_t *ncurve, int *nbcfield);
/* Corner coordinates xc, yc, zc (2^ndim per element, file order; zc may be
 * null for ndim = 2) and the element groups (may be null). */
int nekmesh_re2_xyz(const int64_t *mesh, double *xc, double *yc, double *zc, int *group);
/* The curved-side records: element (1-based), side, the 5 curve values and
 * the curve type character; any output may be null. */
int nekmesh_re2_curves(const int64_t *mesh, int *elem, int *side, double *curve, char *ccurve);
/* Boundary-condition section *field (0-based, in file order) as the
 * reference's dense arrays: cbc[(e*2ndim + f)*3 .. +3] the 3-character type
 * ("E  " where the file has no record), bc[(e*2ndim + f)*5 .. +5] its values
 * (0 where no record). */
int nekmesh_re2_bc(const int64_t *mesh, const int *field, char *cbc, double *bc);
int nekmesh_re2_close(int64_t *mesh);

/* ---- .co2 (core/map2.f read_con :327-471) --------------------------------- */
/* Reads the header (132 bytes: #v001 fixed format a5,3i12 or #v002 free
 * format: nelgt nelgv nv), the byte-order test value and the records (element
 * id and nv vertex ids, 4-byte integers).  vertex (nv * nelgt, element-major,
 * placed by element id) may be null to query the sizes. */
int nekmesh_co2_read(const char *path, int *nelgt, int *nelgv, int *nv, int64_t *vertex);
/* .ma2 map file (core/map2.f read_map :712-940; written by tools/genmap
 * dmp_mapfile): 132-byte header (a5,7i12: version, nel, ...), the byte-order
 * test value, then per element its partition (0-based) and its vertex ids
 * (4-byte integers, tensor corner order, used as read).  vertex (nv * nel)
 * and part (nel) may be null to query the sizes; nv is 8 (or 4 in 2-D). */
int nekmesh_ma2_read(const char *path, int *nel, int *nv, int64_t *vertex, int *part);
/* Writes a #v001 .co2 file, as tools/gencon dmpfile does. */
int nekmesh_co2_write(const char *path, const int *nelgt, const int *nelgv, const int *nv,
                      const int64_t *vertex);

/* ---- connectivity from coordinates (tools/gencon/gencon.f) ----------------- */
/* Global vertex ids (tensor corner order, 1-based, ranked) of nel elements in
 * ndim = 3 from their corners (file order): corners closer than tol times
 * the smaller of their elements' shortest corner-to-neighbour distance are one
 * vertex (unique_vertex2 :1708-1812, set_d2 :308-343; tol 0.2 is gencon's
 * default); faces sharing three vertices with a neighbour get the fourth
 * (face_chk :1827-1925); faces of type "P  " in cbc/bc (the first
 * boundary-condition section, preprocessor face order; may be null) are
 * joined with the face their bc values name (periodic_vtx :1296-1411,
 * find_connctd_pairs :1413-1540).  Fails with NEKGPU_EINVAL when an element
 * ends up with a repeated vertex (self_chk) or a periodic face pair does not
 * match. */
int nekmesh_connect(const int *nel, const int *ndim, const double *xc, const double *yc,
                    const double *zc, const char *cbc, const double *bc, const double *tol,
                    int64_t *vertex, int64_t *nvert);

/* ---- global numbering (core/navier8.f setvert3d :2004-2183) ---------------- */
/* glo_num (nx^3 per element) of nel elements from their vertex ids (tensor
 * corner order): vertices keep their ids, edge and face interiors are
 * numbered by the ranked edges and faces in the reference's orientation,
 * element interiors get 0; *ngv = the number of ids used. */
int nekmesh_setvert3d(const int *nx, const int *nel, const int64_t *vertex, int64_t *glo_num,
                      int64_t *ngv);

/* Single-element periodicity (check_p_bc, core/navier8.f:2571-2620): an
 * element whose two opposite faces both have type "p  " in cbc (preprocessor
 * face order, 6 per element) gets, point by point across the element, the
 * smaller of the two faces' ids on both; set_vert applies it after
 * setvert3d. */
int nekmesh_check_p_bc(const int *nx, const int *nel, const char *cbc, int64_t *glo_num);

/* ---- GLL coordinates of straight-sided elements (core/genxyz.f xyzlin) ---- */
/* x, y, z (nx^3 per element) by the trilinear map of the corners xc, yc, zc
 * (file order) at the GLL nodes zgll[0..nx-1] (xyzlin :1269-1320). */
int nekmesh_xyzlin(const int *nx, const int *nel, const double *zgll, const double *xc,
                   const double *yc, const double *zc, double *x, double *y, double *z);

/* ---- GLL coordinates of curved elements (core/genxyz.f genxyz :558) ----- */
/* As nekmesh_xyzlin for elements without curved sides; an element with a
 * midside-node record (type 'm' on edge 1..12, the 3 node coordinates in
 * curve[5q .. 5q+2]) gets xyzquad's map (:1334-1380): its trilinear 3x3x3
 * nodes, the given midside nodes on their edges, the edges extended inward
 * by Gordon-Hall (gh_face_extend_3d, core/navier5.f:2502, vertices and
 * edges), then the quadratic interpolant at the GLL nodes (Fornberg weights,
 * fd_weights_full, core/fast3d.f:1294; tensr3, core/fasts.f:125).  Then,
 * element by element as genxyz does: every spherical-face record (type 's'
 * on face 1..6, centre in curve[5q .. 5q+2], radius in curve[5q+3]) makes
 * the face a sphere patch as sphsrf does (core/genxyz.f:677-842: great-circle
 * edges, crossings of opposite-edge arcs inside, the deflection spread
 * linearly from the opposite face), then every circular-arc record (type
 * 'C' on edge 1..8, signed radius in curve[5q]; positive with the centre on
 * the element's side) bends its edge as arcsrf does (:2-101), the bend
 * blended linearly across the element.  Records of any other curve type
 * ('e' surfaces) give NEKGPU_EINVAL, as do an arc shorter in radius than
 * half its chord and a sphere corner off its sphere; records with a blank
 * type are ignored.  nx = 2 ignores midside nodes, as linquad. */
int nekmesh_genxyz(const int *nx, const int *nel, const double *zgll, const double *xc,
                   const double *yc, const double *zc, const int64_t *ncurve, const int *elem,
                   const int *side, const double *curve, const char *ccurve, double *x, double *y,
                   double *z);

/* ---- pressure preconditioner setup data (core/hsmg.f; host only) -------- */
/* Level orders of h1mg_setup_mg_nx (:2272-2338): order[0..lmax-1], coarsest
 * first; returns lmax (2 or 3) or NEKGPU_EINVAL (3 <= lx1 <= 12). */
int nekmesh_h1mg_levels(const int *lx1, int *order);
/* Face types as get_fast_bc gives them for the pressure, read from the
 * numbering and mask: per element r-, r+, s-, s+, t-, t+; 0 when the face's
 * point (1, 1) is shared with another element, else 1 when masked, else 2. */
int nekmesh_face_types(const int *nx, const int *nel, const int64_t *glo_num, const double *mask,
                       int *fbc);
/* The setup nekgpu_h1mg_setup computes for level *level (0 = coarsest):
 * *nx its points per direction; its mask, restriction weights (1 /
 * multiplicity) and Schwarz weights (1 / overlap count; 0 on level 0), each
 * nx^3 nel; lengths (may be null): per element the widths of the
 * neighbours and of the element (swap_lengths, core/fast3d.f:1542), 9 per
 * element: left r s t, middle r s t, right r s t. */
int nekmesh_h1mg_level(const int *nx1, const int *nel, const int64_t *glo_num, const double *x,
                       const double *y, const double *z, const double *mask, const int *fbc,
                       const int *level, int *nx, double *lmask, double *rwt, double *swt,
                       double *lengths);
/* One 1-D fast-diagonalisation operator of order n (hsmg_setup_fast1d,
 * core/hsmg.f:783-881) for face types lbc, rbc and widths ll, lm, lr: s the
 * (n+3)^2 eigenvectors (column-major, column j = vector j, rows of excluded
 * points zeroed), lam the n+3 eigenvalues ascending. */
int nekmesh_fdm1d(const int *n, const int *lbc, const int *rbc, const double *ll,
                  const double *lm, const double *lr, double *s, double *lam);

/* The coarse solve's factor A^-1 = X X^T (crs_xxt's form, core/crs_xxt.c:
 * 863): A symmetric positive definite, n x n in CSR (ptr n+1, idx, val,
 * both triangles), its unknowns at xyz (3 each) for the nested-dissection
 * order.  *nnz = the entries of X; with the outputs non-null: perm (n, the
 * unknown numbered k), and X by columns in that order (cptr n+1, cidx and
 * cval nnz: rows of column j). */
int nekmesh_xxt_factor(const int64_t *n, const int64_t *ptr, const int *idx, const double *val,
                       const double *xyz, int64_t *nnz, int *perm, int64_t *cptr, int *cidx,
                       double *cval);

/* The algebraic multigrid hierarchy of a coarse matrix (the reference's
 * crs_amg data, core/crs_amg.c:96-128, which its setup tool writes to amg*.dat
 * files; built here without them): the same setup nekgpu_crs_amg_setup and
 * the AMG coarse solve of the pressure preconditioner run.  A symmetric
 * positive definite, n x n in CSR (ptr n+1, idx, val, both triangles,
 * columns ascending); *plan receives an id for the calls below. */
int nekmesh_amg_setup(const int64_t *n, const int64_t *ptr, const int *idx, const double *val,
                      int64_t *plan);
/* Levels (*nlev), level offsets off (nlev+1: level l holds its F points at
 * [off[l], off[l+1]) of the plan's order) and perm (n: the unknown at each
 * position), each when non-null. */
int nekmesh_amg_layout(const int64_t *plan, int *nlev, int64_t *off, int64_t *perm);
/* Level *lev: sizes[6] = nf, nc and the entries of W, W^T, AfP, A_FF (AfP =
 * A_FF W + A_FC, the F rows of A P with P = [W; I], crs_amg's AfP);
 * Chebyshev steps and radius; the scaled inverse diagonal dff (nf) and the
 * four matrices in CSR (W and AfP: nf rows, W^T: nc rows, A_FF: nf rows),
 * each array when non-null. */
int nekmesh_amg_level(const int64_t *plan, const int *lev, int64_t *sizes, int *m, double *rho,
                      double *dff, int64_t *w_ptr, int *w_idx, double *w_val, int64_t *wt_ptr,
                      int *wt_idx, double *wt_val, int64_t *afp_ptr, int *afp_idx,
                      double *afp_val, int64_t *aff_ptr, int *aff_idx, double *aff_val);
/* One V-cycle (amg_exec, core/crs_amg.c:129-186) on the host, in the plan's
 * order (x out, b overwritten). */
int nekmesh_amg_apply(const int64_t *plan, double *x, double *b);
int nekmesh_amg_free(int64_t *plan);

#ifdef __cplusplus
}
#endif
#endif
