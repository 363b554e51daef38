/* The PLASMA enumerations the reference uses.  Their values equal the CBLAS
 * enumerations, which the reference relies on when it casts them
 * (Hybrid_make_Q.c:30,35-36).  TEST INFRASTRUCTURE ONLY. */
#ifndef HQR_SHIM_PLASMA_H
#define HQR_SHIM_PLASMA_H
#define PLASMA_SUCCESS 0
#define PlasmaNoTrans 111
#define PlasmaTrans 112
#define PlasmaUpper 121
#define PlasmaLower 122
#define PlasmaNonUnit 131
#define PlasmaUnit 132
#define PlasmaLeft 141
#define PlasmaRight 142
#define PlasmaForward 391
#define PlasmaBackward 392
#define PlasmaColumnwise 401
#define PlasmaRowwise 402
static inline char hqr_shim_lapack_const(int c)
{
    switch (c) {
    case PlasmaNoTrans: return 'N';
    case PlasmaTrans: return 'T';
    case PlasmaUpper: return 'U';
    case PlasmaLower: return 'L';
    case PlasmaNonUnit: return 'N';
    case PlasmaUnit: return 'U';
    case PlasmaLeft: return 'L';
    case PlasmaRight: return 'R';
    case PlasmaForward: return 'F';
    case PlasmaBackward: return 'B';
    case PlasmaColumnwise: return 'C';
    case PlasmaRowwise: return 'R';
    default: return '?';
    }
}
#define lapack_const(c) hqr_shim_lapack_const(c)
#endif
