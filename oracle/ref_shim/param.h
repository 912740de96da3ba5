/* Parameter shim used only to compile the reference's own table reader and
 * spline (code/read_tables.cpp, code/spline.cpp) from where they lie, for the
 * oracle cross-checks.  It stands in for code/param.h and supplies the names
 * those two files and their headers use; the values come from -D flags:
 *   REF_GREY (0 ck, 2 particles), REF_IMAX/JMAX/KMAX, REF_GRID_NUM, REF_LX.. */
#ifndef ORACLE_REF_SHIM_PARAM_H
#define ORACLE_REF_SHIM_PARAM_H
#ifndef REF_GREY
#define REF_GREY 0
#endif
#ifndef REF_IMAX
#define REF_IMAX 64
#endif
#ifndef REF_JMAX
#define REF_JMAX 64
#endif
#ifndef REF_KMAX
#define REF_KMAX 64
#endif
#ifndef REF_GRID_NUM
#define REF_GRID_NUM 5
#endif
#ifndef REF_LX
#define REF_LX 1.f
#endif
#ifndef REF_LY
#define REF_LY 1.f
#endif
#ifndef REF_LZ
#define REF_LZ 1.f
#endif
#define num_gpu 1
#define p_row 1
#define imax REF_IMAX
#define jmax REF_JMAX
#define kmax REF_KMAX
#define Lx REF_LX
#define Ly REF_LY
#define Lz REF_LZ
#define grid_num REF_GRID_NUM
#define srt 0
#define grey REF_GREY
#define floatingpoint 0
#define stefan 5.670373e-08
#define pi 3.14159265358979323846
#define myfloat float
#define reade "%e"
#define readf "%f"
#define myfloatF float
#define idx_T(i,j,k,im,jm) ({ i + (im+2)*( j + k*(jm+2) ) ; })
#define pow3(a) ({ a*a*a ; })
#define pow4(a) ({ a*a*a*a ; })
#endif
