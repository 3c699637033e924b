/*
 * Layout-compatible declarations of the IGAP4 plugin structs the GPU glue
 * reads.  Field order and types must stay identical to the reference's
 * include/physimpl.h:13-28 (struct __Phys), include/meshimpl.h:6-29
 * (struct __Mesh), include/bcimpl.h:8-15 (struct __BC),
 * include/commimpl.h:6-17 (struct __Comm) and include/coreimpl.h:11-19
 * (struct __Core), because the glue receives pointers to objects built by
 * IGAP4 itself.  When IGAP4's own headers are included first (building the
 * glue inside IGAP4) these declarations are skipped.
 */
#ifndef IGAPGPU_IGAP_TYPES_H
#define IGAPGPU_IGAP_TYPES_H

#if !defined(COREIMPL)
typedef void (*residual_ptr)(double *residual_, double *u, double *par);
typedef void (*tangent_ptr)(double *tangent_, double *u, double *par);
typedef void (*field_ptr)(double *field, double *u, double *par);
typedef void (*density_ptr)(double h[], double u[], double *par);
typedef void (*densityb_ptr)(double h[], double u[], double traction, double *par, int order);
typedef void (*assert_par_mat_ptr)(double *par);
typedef void (*neumann_ptr)(double *neumann_, double par_neumann[], int face_id, int bc_order, int idof,
                            double xq[]);

struct __Phys {
  int ndim;
  int ndof;
  int torder;
  int sorder;
  double *par_mat;
  int ndensity;
  int nfield;
  residual_ptr residual;
  tangent_ptr tangent;
  field_ptr field;
  density_ptr density;
  densityb_ptr densityb;
  assert_par_mat_ptr assert_par_mat;
};
typedef struct __Phys *Phys;

struct __Mesh {
  int porder;
  int *nelem;
  int *nbasis;
  int *nknot;
  double **knotVector;
  double *wVector;
  double *XVector;
  int nboun;
  int *boun;
  int nsendPart;
  int *sendPart;
  int nrecvPart;
  int *recvPart;
  int *sendBlock;
  int *recvBlock;
  int *universalIdx_temp;
  int *bc_periodic;
  int *nelem_global;
  double **knotVector_global;
  double *wVector_global;
  double *XVector_global;
};
typedef struct __Mesh *Mesh;

struct __BC {
  int *bc_type;
  double *par_periodic;
  double *par_dirichlet;
  double *par_neumann;
  neumann_ptr neumann;
};
typedef struct __BC *BC;

struct __Comm {
  int nselfIdx;
  int *selfIdx;
  int nsendIdx;
  int *sendIdx;
  int *sendPtr;
  int nrecvIdx;
  int *recvIdx;
  int *recvPtr;
  int *globalIdx;
};
typedef struct __Comm *Comm;

struct __Core {
  Phys *phys;
  Mesh *mesh;
  BC *bc;
  Comm *comm;
  double *U_hist;
};
typedef struct __Core *Core;
#endif

#endif
