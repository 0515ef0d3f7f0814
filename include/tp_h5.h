/*
 * tp_h5.h -- the reference's HDF5 files, read and written by libtpgpu.so
 * without libhdf5 (the file format's earliest version, the one libhdf5 writes
 * by default and the reference's files use: version 0/1 superblock, version 1
 * object headers, symbol-table groups, contiguous, compact or chunked
 * datasets, chunks through deflate (the system's zlib, loaded at run time),
 * shuffle and Fletcher-32).  Files in the newer format, or with other filters,
 * are refused with the reason in tp_last_error().
 *
 * Reference locations are paths inside the reference project.
 */
#ifndef TP_H5_H
#define TP_H5_H
#include "tp_types.h"

#ifdef __cplusplus
extern "C" {
#endif

/* --- data_io.c (include/data_io.h:1-15, src/data_io.c:22-120), same names and
 * meaning; hsize_t is a 64-bit unsigned integer.  A program linked against the
 * library needs neither data_io.o nor libhdf5 for its field files.  The HDF5
 * readers read the hyperslab [offset, offset + count) of gname/dset_name (rank
 * dimensions) converted to the memory type; on failure they print the reason
 * (libhdf5 prints its error stack) and leave data untouched.  The binary
 * readers read `size` values from value `offset` on; a missing file is an
 * error (message, exit(1)), as in the reference. */
void read_data_serial_double_h5(int rank, unsigned long long *count, unsigned long long *offset,
                                char *fname, char *gname, char *dset_name, double *data);
void read_data_serial_float_h5(int rank, unsigned long long *count, unsigned long long *offset,
                               char *fname, char *gname, char *dset_name, float *data);
void read_data_serial_float_binary(char *fname, long offset, long size, float *data);
void read_data_serial_double_binary(char *fname, long offset, long size, double *data);

/* The same HDF5 read with a status: elem_bytes 4 (float) or 8 (double).
 * Returns 0, or -1 with tp_last_error() set. */
int tp_h5_read(const char *fname, const char *gname, const char *dset, int rank,
               const unsigned long long *count, const unsigned long long *offset, int elem_bytes,
               void *data);
/* A dataset's rank, dimensions (dims[rank], rank <= 32) and element type
 * (class 0 integer, 1 floating point, 6 compound, -1 other; size in bytes). */
int tp_h5_info(const char *fname, const char *gname, const char *dset, int *rank,
               unsigned long long *dims, int *type_class, int *type_size);

/* --- particles_fields files (save_particles_fields, src/diagnostics.c:290-387;
 * read_particles, src/particle_info.c:376-443): /particles_fields/particles
 * [ntot] compound {x,y,z,qm,ux,uy,uz,t} and /particles_fields/fields [ntot]
 * compound {Bx,By,Bz,Ex,Ey,Ez}, big-endian doubles.  Each rank passes its own
 * records, which go to [naccumulate[mpi_rank - 1], + nptl) (from 0 on rank 0);
 * the file is complete when every rank has returned (the layout depends only
 * on ntot, so the ranks need no exchange).  The fields are the library's FP64
 * get_emf at each record's (x, y, z, t), on the GPU.  system_type is unused,
 * as in the reference.  Returns 0, or -1 with tp_last_error() set. */
int tp_save_particles_fields(int mpi_rank, int nptl, particles *ptl, int ntot, int *naccumulate,
                             char *fname, int system_type);
/* Records [nptl_accumulate[mpi_rank - 1], + nptl) of /particles_fields/particles
 * into x, y, z, qm, ux, uy, uz and t of ptl (the shifts are left as they are),
 * from a file written by the reference or by this library. */
int tp_read_particles(int mpi_rank, int nptl, int *nptl_accumulate, particles *ptl, char *fname);
/* The writer alone, with the fields given (no GPU): records [offset, offset +
 * nptl) of ntot; write_meta on exactly one of the ranks writing the file. */
int tp_h5_write_particles_fields(const char *fname, int write_meta, unsigned long long ntot,
                                 unsigned long long offset, int nptl, const particles *ptl,
                                 const emfields *emf);

/* trajectory_diagnostics (include/diagnostics.h:53-56, src/diagnostics.c:403-568)
 * for one process (mpi_size 1), without MPI or libhdf5: sort by final energy,
 * reload the initial states from data/particles_fields_init.h5, choose
 * nptl_traj_tot particles from the highest energy down, track them again with
 * trajectory records every *nsteps_output steps (particle_tracking_hybrid,
 * traj_diagnose 1) and write data/particle_diagnostics.h5.  Particles of equal
 * energy keep their array order.  Returns 0, or -1 with tp_last_error() set. */
int tp_trajectory_diagnostics(int mpi_rank, int mpi_size, int nptl, double dt, double pmass, int nptl_traj_tot,
                              int system_type, particles *ptl, int *nptl_accumulate, int *nsteps_ptl_tracking,
                              int nbins, int nt_out, int *nsteps_output, int bc_flag, int tracking_method,
                              particles *ptl_init);

/* --- data/poincare_map.h5 (src/poincare_map.c:185-235): /poincare_map/{xpos,
 * ypos,zpos} [npoints_total][ncross + 1] native doubles, this rank's rows
 * [nshift, nshift + npoints) (the rank with nshift 0 writes the metadata).
 * poincare_map's default tp_poincare_save writes this file. */
int tp_h5_write_poincare(const char *fname, int npoints_total, int ncross, int nshift, int npoints,
                         const double *xpos, const double *ypos, const double *zpos);

/* --- PIC field files (read_pic_bfields_float_h5, src/magnetic_field.c:632-692;
 * read_pic_efields_float_h5, src/electric_field.c:447-507): the [nx][ny][nz]
 * datasets cbx, cby, cbz (and ex, ey, ez when with_e) of group gname, float
 * or double, read from the origin, transposed to the reference's x-fastest
 * records and scaled by B0 (E0), straight into device memory, as
 * tp_read_pic_fields_binary does for the .gda files: the values equal the
 * reference's float records bit for bit (file doubles are first rounded to
 * float, as its H5Dread with a float memory type does).  One time frame
 * (multi_tframe 0).  Without with_e the E records are zero. */
int tp_read_pic_fields_h5(const char *fname, const char *gname, int with_e);
/* The inverse: the device-resident PIC fields (tp_synth_pic_fields,
 * tp_read_pic_fields_*) written as such a file, group gname (one level),
 * float datasets cbx, cby, cbz (and ex, ey, ez when with_e) of the records
 * divided by B0 (E0), reordered to C order on the GPU; exact round trips
 * through tp_read_pic_fields_h5 when B0 and E0 are powers of two. */
int tp_save_pic_fields_h5(const char *fname, const char *gname, int with_e);

#ifdef __cplusplus
}
#endif
#endif /* TP_H5_H */
