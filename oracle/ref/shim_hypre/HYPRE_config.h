/* Configuration header for compiling HYPRE's struct solvers from their sources without HYPRE's own
 * build system (oracle/build_hypre.sh): serial (no MPI, HYPRE's MPI stubs), double precision, 32-bit
 * indices, host memory only, HYPRE's bundled BLAS/LAPACK.  Written for this project; it stands in for
 * the header HYPRE's configure step generates. */
#define HYPRE_RELEASE_NAME    "hypre"
#define HYPRE_RELEASE_VERSION "2.33.0"
#define HYPRE_RELEASE_NUMBER  23300
#define HYPRE_RELEASE_DATE    "2025/04/03"
#define HYPRE_RELEASE_TIME    "00:00:00"
#define HYPRE_RELEASE_BUGS    "none"
#define HYPRE_MAXDIM 3
#define HYPRE_SEQUENTIAL 1
#define HYPRE_USING_HYPRE_BLAS 1
#define HYPRE_USING_HYPRE_LAPACK 1
#define HYPRE_USING_HOST_MEMORY 1
#define HYPRE_FMANGLE 0
#define HYPRE_FMANGLE_BLAS 0
#define HYPRE_FMANGLE_LAPACK 0
#define HYPRE_F77_FUNC(name,NAME) name ## _
#define HYPRE_F77_FUNC_(name,NAME) name ## __
