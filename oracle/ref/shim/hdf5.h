/* No-op HDF5 stand-in used only to compile the reference sources for the
 * parity oracle (oracle/_ref).  Every call succeeds and writes nothing; the
 * oracle harness reads results from the objects, not from files. */
#ifndef ORACLE_HDF5_STUB_H
#define ORACLE_HDF5_STUB_H
typedef long long hid_t;
typedef unsigned long long hsize_t;
typedef int herr_t;
typedef int htri_t;
typedef struct { hsize_t nlinks; } H5G_info_t;
#define H5P_DEFAULT 0
#define H5F_ACC_EXCL 0
#define H5F_ACC_RDONLY 0
#define H5F_ACC_RDWR 0
#define H5S_ALL 0
#define H5T_NATIVE_UINT 0
#define H5T_STD_U32BE 0
#define ORACLE_H5_NOOP(name) template <class... A> inline hid_t name(A...) { return 0; }
ORACLE_H5_NOOP(H5Aclose)
ORACLE_H5_NOOP(H5Acreate)
ORACLE_H5_NOOP(H5Awrite)
ORACLE_H5_NOOP(H5Dclose)
ORACLE_H5_NOOP(H5Dget_type)
ORACLE_H5_NOOP(H5Dopen)
ORACLE_H5_NOOP(H5Dopen2)
ORACLE_H5_NOOP(H5Dwrite)
ORACLE_H5_NOOP(H5Fclose)
ORACLE_H5_NOOP(H5Fcreate)
ORACLE_H5_NOOP(H5Fopen)
ORACLE_H5_NOOP(H5Gclose)
ORACLE_H5_NOOP(H5Gcreate)
ORACLE_H5_NOOP(H5Gcreate2)
ORACLE_H5_NOOP(H5Gopen)
ORACLE_H5_NOOP(H5LTmake_dataset_double)
ORACLE_H5_NOOP(H5LTmake_dataset_int)
ORACLE_H5_NOOP(H5LTread_dataset_int)
ORACLE_H5_NOOP(H5LTset_attribute_double)
ORACLE_H5_NOOP(H5LTset_attribute_string)
ORACLE_H5_NOOP(H5Lexists)
ORACLE_H5_NOOP(H5Sclose)
ORACLE_H5_NOOP(H5Screate_simple)
ORACLE_H5_NOOP(H5Tclose)
ORACLE_H5_NOOP(H5close)
inline herr_t H5Gget_info_by_name(hid_t, const char*, H5G_info_t* info, hid_t)
{
    info->nlinks = 0;
    return 0;
}
#undef ORACLE_H5_NOOP
#endif
