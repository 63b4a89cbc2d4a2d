/*
 * Test double of libtrexio for the TREXIO reader's tests (test infrastructure, not shipped).
 *
 * It implements the part of TREXIO's C API that the reader binds (trexio_open, trexio_close,
 * trexio_string_of_error, the *_num_64 attributes, trexio_read_basis_type and the
 * trexio_read_safe_*_64/_32 datasets) over a file format of its own, written by files.py beside
 * this file:
 *
 *   8 bytes  "TRXDBL1" + back-end letter ('T' opens with the text back end, 'H' with HDF5)
 *   records  char name[48] (NUL-padded, e.g. "basis_nucleus_index"), int32 kind (1 int64,
 *            2 double, 3 int32, 4 string), int32 pad, int64 count, count elements (strings:
 *            count bytes)
 *
 * Exit codes follow TREXIO's convention that 0 is success; the nonzero values are this double's.
 * Calls are counted per entry point (trexio_double_calls) so that a test can see which back ends
 * were tried.
 */
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

typedef int32_t trexio_exit_code;
typedef int32_t back_end_t;
typedef struct trexio_s trexio_t;

enum {
  DBL_SUCCESS = 0,
  DBL_INVALID_ARG_1 = 1,
  DBL_INVALID_ARG_2 = 2,
  DBL_INVALID_ARG_3 = 3,
  DBL_OPEN_ERROR = 19,
  DBL_HAS_NOT = 15,
  DBL_UNSAFE_ARRAY_DIM = 23,
  DBL_WRONG_KIND = 40,
  DBL_CORRUPT = 41
};

enum { KIND_INT64 = 1, KIND_DOUBLE = 2, KIND_INT32 = 3, KIND_STRING = 4 };

struct record {
  char name[49];
  int32_t kind;
  int64_t count;
  unsigned char* data;
};

struct trexio_s {
  int n;
  struct record* rec;
};

static int64_t calls_open_text, calls_open_hdf5, calls_close;

int64_t trexio_double_calls(int which) {
  return which == 0 ? calls_open_text : which == 1 ? calls_open_hdf5 : calls_close;
}

static size_t elem_size(int32_t kind) {
  return kind == KIND_INT64 || kind == KIND_DOUBLE ? 8 : kind == KIND_INT32 ? 4 : 1;
}

static void release(trexio_t* f) {
  if (!f) return;
  for (int i = 0; i < f->n; ++i) free(f->rec[i].data);
  free(f->rec);
  free(f);
}

trexio_t* trexio_open(const char* file_name, const char mode, const back_end_t back_end, trexio_exit_code* const rc) {
  if (back_end == 1) ++calls_open_text;
  if (back_end == 0) ++calls_open_hdf5;
  trexio_exit_code dummy;
  trexio_exit_code* out = rc ? rc : &dummy;
  if (!file_name) { *out = DBL_INVALID_ARG_1; return NULL; }
  if (mode != 'r') { *out = DBL_INVALID_ARG_2; return NULL; }
  FILE* fp = fopen(file_name, "rb");
  if (!fp) { *out = DBL_OPEN_ERROR; return NULL; }
  char magic[8];
  if (fread(magic, 1, 8, fp) != 8 || memcmp(magic, "TRXDBL1", 7) != 0) {
    fclose(fp);
    *out = DBL_OPEN_ERROR;
    return NULL;
  }
  const char want = back_end == 1 ? 'T' : back_end == 0 ? 'H' : '?';
  if (magic[7] != want) {
    fclose(fp);
    *out = DBL_OPEN_ERROR;
    return NULL;
  }
  trexio_t* f = (trexio_t*)calloc(1, sizeof *f);
  if (!f) { fclose(fp); *out = DBL_OPEN_ERROR; return NULL; }
  for (;;) {
    char name[48];
    size_t got = fread(name, 1, 48, fp);
    if (got == 0) break;
    int32_t kind, pad;
    int64_t count;
    if (got != 48 || fread(&kind, 4, 1, fp) != 1 || fread(&pad, 4, 1, fp) != 1 || fread(&count, 8, 1, fp) != 1 ||
        kind < KIND_INT64 || kind > KIND_STRING || count < 0 || count > ((int64_t)1 << 32)) {
      release(f);
      fclose(fp);
      *out = DBL_CORRUPT;
      return NULL;
    }
    struct record* grown = (struct record*)realloc(f->rec, sizeof(struct record) * (size_t)(f->n + 1));
    if (!grown) { release(f); fclose(fp); *out = DBL_CORRUPT; return NULL; }
    f->rec = grown;
    struct record* r = &f->rec[f->n];
    memset(r, 0, sizeof *r);
    memcpy(r->name, name, 48);
    r->kind = kind;
    r->count = count;
    size_t bytes = (size_t)count * elem_size(kind);
    r->data = (unsigned char*)malloc(bytes ? bytes : 1);
    f->n += 1;
    if (!r->data || fread(r->data, 1, bytes, fp) != bytes) {
      release(f);
      fclose(fp);
      *out = DBL_CORRUPT;
      return NULL;
    }
  }
  fclose(fp);
  *out = DBL_SUCCESS;
  return f;
}

trexio_exit_code trexio_close(trexio_t* file) {
  ++calls_close;
  if (!file) return DBL_INVALID_ARG_1;
  release(file);
  return DBL_SUCCESS;
}

const char* trexio_string_of_error(const trexio_exit_code error) {
  switch (error) {
    case DBL_SUCCESS: return "Success";
    case DBL_INVALID_ARG_1: return "Invalid argument 1";
    case DBL_INVALID_ARG_2: return "Invalid argument 2";
    case DBL_INVALID_ARG_3: return "Invalid argument 3";
    case DBL_OPEN_ERROR: return "Error opening file";
    case DBL_HAS_NOT: return "Element absent";
    case DBL_UNSAFE_ARRAY_DIM: return "Incorrect array dimensions";
    case DBL_WRONG_KIND: return "Element of another type";
    case DBL_CORRUPT: return "Corrupt file";
    default: return "Unknown error";
  }
}

static const struct record* find(const trexio_t* f, const char* name) {
  for (int i = 0; i < f->n; ++i)
    if (strcmp(f->rec[i].name, name) == 0) return &f->rec[i];
  return NULL;
}

static trexio_exit_code read_num(trexio_t* const f, const char* name, int64_t* const num) {
  if (!f) return DBL_INVALID_ARG_1;
  if (!num) return DBL_INVALID_ARG_2;
  const struct record* r = find(f, name);
  if (!r) return DBL_HAS_NOT;
  if (r->kind != KIND_INT64 || r->count != 1) return DBL_WRONG_KIND;
  memcpy(num, r->data, 8);
  return DBL_SUCCESS;
}

static trexio_exit_code read_dset(trexio_t* const f, const char* name, int32_t kind, void* const out, int64_t dim) {
  if (!f) return DBL_INVALID_ARG_1;
  if (!out) return DBL_INVALID_ARG_2;
  const struct record* r = find(f, name);
  if (!r) return DBL_HAS_NOT;
  if (r->kind != kind) return DBL_WRONG_KIND;
  if (dim != r->count) return DBL_UNSAFE_ARRAY_DIM;
  memcpy(out, r->data, (size_t)r->count * elem_size(kind));
  return DBL_SUCCESS;
}

#define NUM(fn, key) \
  trexio_exit_code fn(trexio_t* const file, int64_t* const num) { return read_num(file, key, num); }
NUM(trexio_read_electron_up_num_64, "electron_up_num")
NUM(trexio_read_electron_dn_num_64, "electron_dn_num")
NUM(trexio_read_nucleus_num_64, "nucleus_num")
NUM(trexio_read_basis_shell_num_64, "basis_shell_num")
NUM(trexio_read_basis_prim_num_64, "basis_prim_num")
NUM(trexio_read_ao_num_64, "ao_num")
NUM(trexio_read_mo_num_64, "mo_num")

#define DSET(fn, key, T, kind)                                                   \
  trexio_exit_code fn(trexio_t* const file, T* const dset_out, const int64_t dim_out) { \
    return read_dset(file, key, kind, dset_out, dim_out);                        \
  }
DSET(trexio_read_safe_nucleus_charge_64, "nucleus_charge", double, KIND_DOUBLE)
DSET(trexio_read_safe_nucleus_coord_64, "nucleus_coord", double, KIND_DOUBLE)
DSET(trexio_read_safe_basis_nucleus_index_64, "basis_nucleus_index", int64_t, KIND_INT64)
DSET(trexio_read_safe_basis_shell_ang_mom_32, "basis_shell_ang_mom", int32_t, KIND_INT32)
DSET(trexio_read_safe_basis_shell_factor_64, "basis_shell_factor", double, KIND_DOUBLE)
DSET(trexio_read_safe_basis_shell_index_64, "basis_shell_index", int64_t, KIND_INT64)
DSET(trexio_read_safe_basis_exponent_64, "basis_exponent", double, KIND_DOUBLE)
DSET(trexio_read_safe_basis_coefficient_64, "basis_coefficient", double, KIND_DOUBLE)
DSET(trexio_read_safe_basis_prim_factor_64, "basis_prim_factor", double, KIND_DOUBLE)
DSET(trexio_read_safe_ao_normalization_64, "ao_normalization", double, KIND_DOUBLE)
DSET(trexio_read_safe_mo_coefficient_64, "mo_coefficient", double, KIND_DOUBLE)

trexio_exit_code trexio_read_basis_type(trexio_t* const file, char* const str, const int32_t max_str_len) {
  if (!file) return DBL_INVALID_ARG_1;
  if (!str) return DBL_INVALID_ARG_2;
  if (max_str_len <= 0) return DBL_INVALID_ARG_3;
  const struct record* r = find(file, "basis_type");
  if (!r) return DBL_HAS_NOT;
  if (r->kind != KIND_STRING) return DBL_WRONG_KIND;
  size_t n = (size_t)r->count < (size_t)max_str_len - 1 ? (size_t)r->count : (size_t)max_str_len - 1;
  memcpy(str, r->data, n);
  str[n] = '\0';
  return DBL_SUCCESS;
}
