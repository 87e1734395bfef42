/*
 * lgb_io.c -- PETSc binary files in and out of the swarms.
 *
 * Replaces the file side of LagRBF's data ingestion and output: VecLoadFromFile / ISLoadFromFile
 * (src/io_utils.c:211-238), SwarmSetFromPetscFiles / SwarmSetFieldFromPetscFile
 * (src/readers/petsc_loader/petsc_loader.c:38-99), SwarmInterpLoadPidxFromFile
 * (src/swarm/swarm_interp.c:180-222) and SwarmOutputFieldPetscVec/IS_FromName
 * (src/swarm/swarm_output.c:87-166), without PETSc.
 *
 * Format (PETSc binary viewer, 32-bit PetscInt, double PetscScalar, big-endian):
 *   Vec: int32 class id 1211214, int32 n, n doubles
 *   IS:  int32 class id 1211218, int32 n, n int32
 * A Vec's block size travels in the side file "<name>.info" as the line "-vecload_block_size <bs>"
 * (absent: 1), which is where VecLoad takes it from.
 */
#include "lgb_internal.h"
#include "../../include/lagrbf.h"

#include <errno.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#define VEC_CLASSID 1211214
#define IS_CLASSID 1211218

int lgb_set_error_msg(int code, const char *msg);

static int io_error(int code, const char *what, const char *path)
{
  char msg[600];
  snprintf(msg, sizeof(msg), "%s: %s", what, path ? path : "(null)");
  return lgb_set_error_msg(code, msg);
}

static void put_be32(unsigned char *b, uint32_t v)
{
  b[0] = (unsigned char)(v >> 24); b[1] = (unsigned char)(v >> 16); b[2] = (unsigned char)(v >> 8); b[3] = (unsigned char)v;
}
static uint32_t get_be32(const unsigned char *b)
{
  return ((uint32_t)b[0] << 24) | ((uint32_t)b[1] << 16) | ((uint32_t)b[2] << 8) | (uint32_t)b[3];
}
static void put_be64(unsigned char *b, uint64_t v)
{
  int i;
  for (i = 0; i < 8; i++) b[i] = (unsigned char)(v >> (56 - 8 * i));
}
static uint64_t get_be64(const unsigned char *b)
{
  uint64_t v = 0;
  int i;
  for (i = 0; i < 8; i++) v = (v << 8) | b[i];
  return v;
}

/* Block size from "<path>.info" (1 when the file or the key is absent). */
static int read_info_bs(const char *path)
{
  char name[4096], line[512];
  FILE *f;
  int bs = 1;
  snprintf(name, sizeof(name), "%s.info", path);
  f = fopen(name, "r");
  if (!f) return 1;
  while (fgets(line, sizeof(line), f)) {
    char *p = strstr(line, "-vecload_block_size");
    if (p) {
      int v = atoi(p + strlen("-vecload_block_size"));
      if (v > 0) bs = v;
    }
  }
  fclose(f);
  return bs;
}

static int write_header(FILE *f, int classid, int64_t n)
{
  unsigned char h[8];
  put_be32(h, (uint32_t)classid);
  put_be32(h + 4, (uint32_t)n);
  return fwrite(h, 1, 8, f) == 8 ? 0 : -1;
}

static int read_header(FILE *f, int classid, int64_t *n)
{
  unsigned char h[8];
  int32_t cnt;
  if (fread(h, 1, 8, f) != 8) return -1;
  if ((int32_t)get_be32(h) != classid) return -2;
  cnt = (int32_t)get_be32(h + 4);
  if (cnt < 0) return -3;
  *n = cnt;
  return 0;
}

LAGRBF_EXPORT int lagrbf_petsc_vec_write(const char *path, const double *v, int64_t n, int32_t bs)
{
  FILE *f;
  unsigned char buf[8 * 1024];
  int64_t i = 0;
  if (!path || (n > 0 && !v)) return io_error(LAGRBF_ERR_ARG_NULL, "NULL path or values", path);
  if (n < 0 || n > INT32_MAX || bs < 1) return io_error(LAGRBF_ERR_ARG_OUTOFRANGE, "vector length or block size out of range", path);
  f = fopen(path, "wb");
  if (!f) return io_error(LAGRBF_ERR_ARG_WRONG, "cannot open for writing", path);
  if (write_header(f, VEC_CLASSID, n)) { fclose(f); return io_error(LAGRBF_ERR_ARG_WRONG, "write failed", path); }
  while (i < n) {
    int64_t k, c = n - i < 1024 ? n - i : 1024;
    for (k = 0; k < c; k++) {
      uint64_t u;
      memcpy(&u, &v[i + k], 8);
      put_be64(buf + 8 * k, u);
    }
    if (fwrite(buf, 8, (size_t)c, f) != (size_t)c) { fclose(f); return io_error(LAGRBF_ERR_ARG_WRONG, "write failed", path); }
    i += c;
  }
  if (fclose(f)) return io_error(LAGRBF_ERR_ARG_WRONG, "write failed", path);
  {
    char name[4096];
    snprintf(name, sizeof(name), "%s.info", path);
    if (bs > 1) {
      FILE *g = fopen(name, "w");
      if (!g) return io_error(LAGRBF_ERR_ARG_WRONG, "cannot write the .info file of", path);
      fprintf(g, "-vecload_block_size %d\n", bs);
      fclose(g);
    } else {
      remove(name);
    }
  }
  return 0;
}

LAGRBF_EXPORT int lagrbf_petsc_vec_read(const char *path, double *v, int64_t cap, int64_t *n, int32_t *bs)
{
  FILE *f;
  unsigned char buf[8 * 1024];
  int64_t cnt, i = 0;
  int rc;
  if (!path || !n) return io_error(LAGRBF_ERR_ARG_NULL, "NULL path or length", path);
  f = fopen(path, "rb");
  if (!f) return io_error(LAGRBF_ERR_ARG_WRONG, "cannot open", path);
  rc = read_header(f, VEC_CLASSID, &cnt);
  if (rc) {
    fclose(f);
    return io_error(LAGRBF_ERR_ARG_WRONG, rc == -2 ? "not a PETSc binary Vec file" : "truncated PETSc binary file", path);
  }
  *n = cnt;
  if (bs) *bs = read_info_bs(path);
  if (v) {
    if (cap < cnt) { fclose(f); return io_error(LAGRBF_ERR_ARG_SIZ, "buffer smaller than the vector in", path); }
    while (i < cnt) {
      int64_t k, c = cnt - i < 1024 ? cnt - i : 1024;
      if (fread(buf, 8, (size_t)c, f) != (size_t)c) { fclose(f); return io_error(LAGRBF_ERR_ARG_WRONG, "truncated PETSc binary file", path); }
      for (k = 0; k < c; k++) {
        uint64_t u = get_be64(buf + 8 * k);
        memcpy(&v[i + k], &u, 8);
      }
      i += c;
    }
  }
  fclose(f);
  return 0;
}

LAGRBF_EXPORT int lagrbf_petsc_is_write(const char *path, const int64_t *idx, int64_t n)
{
  FILE *f;
  unsigned char buf[4 * 1024];
  int64_t i = 0;
  if (!path || (n > 0 && !idx)) return io_error(LAGRBF_ERR_ARG_NULL, "NULL path or indices", path);
  if (n < 0 || n > INT32_MAX) return io_error(LAGRBF_ERR_ARG_OUTOFRANGE, "index set length out of range", path);
  for (i = 0; i < n; i++)
    if (idx[i] < INT32_MIN || idx[i] > INT32_MAX) /* PetscIntCast to 32-bit PetscInt */
      return io_error(LAGRBF_ERR_ARG_OUTOFRANGE, "index does not fit a 32-bit PetscInt for", path);
  f = fopen(path, "wb");
  if (!f) return io_error(LAGRBF_ERR_ARG_WRONG, "cannot open for writing", path);
  if (write_header(f, IS_CLASSID, n)) { fclose(f); return io_error(LAGRBF_ERR_ARG_WRONG, "write failed", path); }
  i = 0;
  while (i < n) {
    int64_t k, c = n - i < 1024 ? n - i : 1024;
    for (k = 0; k < c; k++) put_be32(buf + 4 * k, (uint32_t)(int32_t)idx[i + k]);
    if (fwrite(buf, 4, (size_t)c, f) != (size_t)c) { fclose(f); return io_error(LAGRBF_ERR_ARG_WRONG, "write failed", path); }
    i += c;
  }
  if (fclose(f)) return io_error(LAGRBF_ERR_ARG_WRONG, "write failed", path);
  return 0;
}

LAGRBF_EXPORT int lagrbf_petsc_is_read(const char *path, int64_t *idx, int64_t cap, int64_t *n)
{
  FILE *f;
  unsigned char buf[4 * 1024];
  int64_t cnt, i = 0;
  int rc;
  if (!path || !n) return io_error(LAGRBF_ERR_ARG_NULL, "NULL path or length", path);
  f = fopen(path, "rb");
  if (!f) return io_error(LAGRBF_ERR_ARG_WRONG, "cannot open", path);
  rc = read_header(f, IS_CLASSID, &cnt);
  if (rc) {
    fclose(f);
    return io_error(LAGRBF_ERR_ARG_WRONG, rc == -2 ? "not a PETSc binary IS file" : "truncated PETSc binary file", path);
  }
  *n = cnt;
  if (idx) {
    if (cap < cnt) { fclose(f); return io_error(LAGRBF_ERR_ARG_SIZ, "buffer smaller than the index set in", path); }
    while (i < cnt) {
      int64_t k, c = cnt - i < 1024 ? cnt - i : 1024;
      if (fread(buf, 4, (size_t)c, f) != (size_t)c) { fclose(f); return io_error(LAGRBF_ERR_ARG_WRONG, "truncated PETSc binary file", path); }
      for (k = 0; k < c; k++) idx[i + k] = (int32_t)get_be32(buf + 4 * k);
      i += c;
    }
  }
  fclose(f);
  return 0;
}

/* Loads a Vec file into a fresh array; *bs its block size. */
static int load_vec(const char *path, double **out, int64_t *n, int32_t *bs)
{
  int rc = lagrbf_petsc_vec_read(path, NULL, 0, n, bs);
  if (rc) return rc;
  *out = (double *)malloc(sizeof(double) * (size_t)(*n > 0 ? *n : 1));
  if (!*out) return io_error(LAGRBF_ERR_MEM, "out of host memory reading", path);
  rc = lagrbf_petsc_vec_read(path, *out, *n, n, bs);
  if (rc) { free(*out); *out = NULL; }
  return rc;
}

int lgb_ctx_dims(void *ctx, int *dim, int *nfields);

LAGRBF_EXPORT int lagrbf_fill_swarm_from_files(void *ctx, bool is_data, const char *coords_file, const char **field_files,
                                               int32_t nfiles, const char *pid_file)
{
  double *coords = NULL, *values = NULL, *v = NULL;
  int64_t *pid = NULL, n = 0, nv = 0, np = 0, p;
  int32_t bs = 1;
  int dim = 0, F = 0, rc, f, pos = 0, b;
  if (!ctx) return lgb_set_error_msg(LAGRBF_ERR_ARG_NULL, "context is NULL");
  if (!coords_file || (nfiles > 0 && !field_files)) return lgb_set_error_msg(LAGRBF_ERR_ARG_NULL, "NULL file name");
  if ((rc = lgb_ctx_dims(ctx, &dim, &F))) return rc;
  /* coordinates set the number of points (SwarmLoadCoordinatesFromFile) */
  if ((rc = load_vec(coords_file, &coords, &nv, &bs))) return rc;
  if (bs != dim && !(bs == 1 && nv % dim == 0)) { rc = io_error(LAGRBF_ERR_ARG_SIZ, "coordinate block size differs from the mesh dimension in", coords_file); goto done; }
  n = nv / dim;
  if (nfiles > 0) {
    values = (double *)calloc((size_t)(n > 0 ? n : 1) * (size_t)(F > 0 ? F : 1), sizeof(double));
    if (!values) { rc = lgb_set_error_msg(LAGRBF_ERR_MEM, "out of host memory"); goto done; }
  }
  /* fields stacked in file order (SwarmSetFieldFromPetscFile) */
  for (f = 0; f < nfiles; f++) {
    int64_t m;
    if ((rc = load_vec(field_files[f], &v, &nv, &bs))) goto done;
    m = nv / bs;
    if (m != n || nv % bs) { rc = io_error(LAGRBF_ERR_ARG_SIZ, "loaded vector size does not match the swarm size for", field_files[f]); goto done; }
    if (pos + bs > F) { rc = io_error(LAGRBF_ERR_ARG_SIZ, "too many fields to load (n_interpolation_fields) from", field_files[f]); goto done; }
    for (p = 0; p < n; p++)
      for (b = 0; b < bs; b++) values[p * F + pos + b] = v[p * bs + b];
    pos += bs;
    free(v);
    v = NULL;
  }
  if (pid_file) {
    if ((rc = lagrbf_petsc_is_read(pid_file, NULL, 0, &np))) goto done;
    if (np != n) { rc = io_error(LAGRBF_ERR_ARG_SIZ, "index set size does not match the swarm size in", pid_file); goto done; }
    pid = (int64_t *)malloc(sizeof(int64_t) * (size_t)(n > 0 ? n : 1));
    if (!pid) { rc = lgb_set_error_msg(LAGRBF_ERR_MEM, "out of host memory"); goto done; }
    if ((rc = lagrbf_petsc_is_read(pid_file, pid, n, &np))) goto done;
  }
  if (n > INT32_MAX) { rc = lgb_set_error_msg(LAGRBF_ERR_ARG_OUTOFRANGE, "too many points for a 32-bit PetscInt"); goto done; }
  rc = lagrbf_fill_swarm(ctx, is_data, (int32_t)n, coords, values, pid);
done:
  free(coords); free(values); free(v); free(pid);
  return rc;
}

LAGRBF_EXPORT int lagrbf_output_files(void *ctx, bool is_data, int32_t nglobal, const char *prefix, const char *fieldname)
{
  double *coords = NULL, *fields = NULL;
  int64_t *pid = NULL;
  int dim = 0, F = 0, nf, rc;
  char name[4096];
  if (!ctx) return lgb_set_error_msg(LAGRBF_ERR_ARG_NULL, "context is NULL");
  if (!prefix) return lgb_set_error_msg(LAGRBF_ERR_ARG_NULL, "NULL prefix");
  if (nglobal <= 0) return lgb_set_error_msg(LAGRBF_ERR_ARG_OUTOFRANGE, "npoints must be positive");
  if ((rc = lgb_ctx_dims(ctx, &dim, &F))) return rc;
  if (!fieldname) fieldname = "fields";
  nf = !strcmp(fieldname, "velocity") ? dim : !strcmp(fieldname, "weights") ? (1 << dim) : F;
  coords = (double *)malloc(sizeof(double) * (size_t)nglobal * dim);
  fields = (double *)malloc(sizeof(double) * (size_t)nglobal * (nf > 0 ? nf : 1));
  pid = (int64_t *)malloc(sizeof(int64_t) * (size_t)nglobal);
  if (!coords || !fields || !pid) { rc = lgb_set_error_msg(LAGRBF_ERR_MEM, "out of host memory"); goto done; }
  rc = lagrbf_output(ctx, is_data, nglobal, coords, nf > 0 ? fields : NULL, pid, fieldname);
  if (rc) goto done;
  snprintf(name, sizeof(name), "%s_coor.pbvec", prefix);
  if ((rc = lagrbf_petsc_vec_write(name, coords, (int64_t)nglobal * dim, dim))) goto done;
  if (nf > 0) {
    snprintf(name, sizeof(name), "%s_%s.pbvec", prefix, fieldname);
    if ((rc = lagrbf_petsc_vec_write(name, fields, (int64_t)nglobal * nf, nf))) goto done;
  }
  snprintf(name, sizeof(name), "%s_pid.pbis", prefix);
  rc = lagrbf_petsc_is_write(name, pid, nglobal);
done:
  free(coords); free(fields); free(pid);
  return rc;
}
