/*
 * kevd_h5.h — the HDF5 datasets the reference's three programs read and write,
 * without libhdf5.
 *
 * The reference moves every array between its stages through HDF5 files:
 *   - the KS states "/u" (float32, ks_bandwidth.cu:51-83 h5read, ks_arpclm.cu:82-115,
 *     ks_kevd.cu:134-170; written by ks_datagen.py:91-103 through h5py);
 *   - the stage-2 outputs "/linv" (float64) and "/spiv" (unsigned 64-bit), written by
 *     ks_arpclm.cu:121-172 (h5write_sizet, h5write_double) and read back by
 *     ks_kevd.cu:113-243 (h5_num_elements, h5read_double, h5read_sizet);
 *   - the stage-3 outputs "/lam" (float64) and "/U" (float32), appended one dataset at a
 *     time to a file created empty (ks_kevd.cu:247-290 h5add_double / h5add_float,
 *     :492-503 H5Fcreate).
 * Every one of those datasets is a one-dimensional array in the root group, stored
 * contiguously.  This library reads and writes exactly that subset of the HDF5 file
 * format (public specification, format versions 0-3 of the superblock):
 *
 *   read:  superblock versions 0-3 (a user block before it is allowed), object headers
 *          versions 1 and 2 with continuation blocks, groups stored as a symbol table
 *          (v1 B-tree, symbol nodes, local heap) or as compact link messages, nested
 *          group paths, contiguous or compact datasets of any rank (read flat, in
 *          storage order) whose elements are IEEE binary32/binary64 or 1/2/4/8-byte
 *          integers of either byte order;
 *   write: superblock version 0 with 8-byte offsets and lengths, a symbol-table root
 *          group, one-dimensional contiguous datasets of float32, float64, int32,
 *          uint32, int64, uint64 (little-endian): the structures libhdf5 writes with its
 *          default ("earliest") format settings (compared with a libhdf5-written file;
 *          no libhdf5 was at hand to read these files back).
 *
 * Chunked or filtered (compressed) datasets, dense (fractal-heap) groups, committed
 * datatypes, external storage and virtual datasets are reported as
 * KEVD_H5_ERR_UNSUPPORTED.  Reading converts to the requested element type as H5Dread
 * does with a native memory type: floating types by C conversion, integer targets
 * clamped to their range.
 *
 * Entry points return KEVD_H5_OK or an error code; kevd_h5_last_error() describes the
 * last failure on the calling thread.  No function keeps a file open between calls.
 * Reads of one file may run concurrently; an append must not overlap any other call on
 * the same file (as with libhdf5 without its thread-safe build).
 */
#ifndef KEVD_H5_H
#define KEVD_H5_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum kevd_h5_status {
    KEVD_H5_OK = 0,
    KEVD_H5_ERR_ARG = 1,          /* bad argument: count mismatch, bad name, duplicate  */
    KEVD_H5_ERR_IO = 2,           /* the file cannot be opened, read or written         */
    KEVD_H5_ERR_FORMAT = 3,       /* not an HDF5 file, or a corrupt structure           */
    KEVD_H5_ERR_NOTFOUND = 4,     /* no dataset of that name                            */
    KEVD_H5_ERR_UNSUPPORTED = 5   /* a valid HDF5 feature outside the subset above      */
};

/* Element types (the reference's H5T_NATIVE_FLOAT, _DOUBLE, _INT, _UINT, _LONG, _ULONG
 * on an LP64 host). */
enum kevd_h5_type {
    KEVD_H5_F32 = 1,
    KEVD_H5_F64 = 2,
    KEVD_H5_I32 = 3,
    KEVD_H5_U32 = 4,
    KEVD_H5_I64 = 5,
    KEVD_H5_U64 = 6
};

const char* kevd_h5_last_error(void);

/* Size, rank and dimensions (up to 32) of dataset `name` ("/u" or "u"; "/g/u" inside
 * group g) and the stored element type as the nearest kevd_h5_type: integers of 1 or 2
 * bytes report I32/U32, a float of 4 bytes F32, of 8 bytes F64.  `count` is the number
 * of elements (the product of the dimensions: ks_kevd.cu:113-132
 * H5Sget_simple_extent_npoints).  Any output pointer may be NULL. */
int kevd_h5_dataset_info(const char* path, const char* name, int64_t* count, int32_t* type,
                         int32_t* rank, int64_t* dims);

/* Reads all `count` elements of dataset `name` into `out`, converted to `type`
 * (ks_bandwidth.cu:51-83 h5read: the caller states the element count it expects and a
 * different count is an error, as the reference asserts it). */
int kevd_h5_read(const char* path, const char* name, int32_t type, void* out, int64_t count);

/* Names of the datasets and groups in the root group, each NUL-terminated, one after
 * another in `buf` (at most `cap` bytes); `n` receives how many. */
int kevd_h5_list(const char* path, char* buf, int64_t cap, int32_t* n);

/* Creates (or truncates) `path` as an HDF5 file with an empty root group
 * (ks_kevd.cu:497-502 H5Fcreate with H5F_ACC_TRUNC). */
int kevd_h5_create(const char* path);

/* Adds the one-dimensional dataset `name` of `count` elements to the root group of an
 * existing file (ks_kevd.cu:247-290 h5add_double / h5add_float).  The data are written
 * after the file's last byte and the root group's index is rewritten; the datasets
 * already there keep their places.  The file must have a version 0 or 1 superblock with
 * 8-byte offsets and lengths and a symbol-table root group (what kevd_h5_create and
 * libhdf5's default settings make).  A name already in the group is KEVD_H5_ERR_ARG. */
int kevd_h5_append(const char* path, const char* name, int32_t type, const void* data, int64_t count);

/* kevd_h5_create followed by kevd_h5_append of each of the `n` datasets
 * (ks_arpclm.cu:121-172 h5write_sizet / h5write_double write one dataset per file). */
int kevd_h5_write(const char* path, int32_t n, const char* const* names, const int32_t* types,
                  const void* const* data, const int64_t* counts);

#ifdef __cplusplus
}
#endif

#endif /* KEVD_H5_H */
