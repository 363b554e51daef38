/* Linked into the shimmed reference build only (TEST INFRASTRUCTURE).  The
 * reference links the sequential OpenBLAS (openblas_seq, Makefile:4); the
 * scipy-bundled OpenBLAS is threaded, so pin it to one thread before use. */
void scipy_openblas_set_num_threads(int n);
__attribute__((constructor)) static void hqr_ref_init(void)
{
    scipy_openblas_set_num_threads(1);
}
