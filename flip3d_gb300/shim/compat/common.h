/*
 * common.h (shim build without the reference tree) — the particle record and
 * constants a flip3d driver passes through the sorter/mapper/solver/
 * corrector interface. The layout must equal the driver's (src/common.h:24-49:
 * p, u, n, four chars, tmp[2][3], m, dens; FLOAT = float) because the shim
 * reads and writes those records in place; a build that has the driver's own
 * common.h uses that one instead.
 */
#ifndef _COMMON_H
#define _COMMON_H

#define FLOAT float
#define AIR 0
#define FLUID 1
#define WALL 2

typedef struct _particle {
  FLOAT p[3];
  FLOAT u[3];
  FLOAT n[3];
  char type;
  char visible;
  char remove;
  char thinparticle;
  FLOAT tmp[2][3];
  FLOAT m;
  FLOAT dens;
} particle;

#endif
