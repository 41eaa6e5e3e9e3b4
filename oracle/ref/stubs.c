/* Test infrastructure: no-op stand-ins for the XSPICE event-driven core,
 * the B-source expression parser and the safe-operating-area checker.  The
 * oracle netlists contain no event-driven ("A") instances, no B sources and
 * no SOA checks, so the reference never reaches these with real work; they
 * only satisfy the linker.  Prototypes are deliberately loose (the linker
 * does not check them) and each returns 0 = OK. */
int EVTop(void) { return 0; }
int EVTdump(void) { return 0; }
int EVTop_save(void) { return 0; }
int EVTiter(void) { return 0; }
int EVTcall_hybrids(void) { return 0; }
double EVTnext_time(void) { return 1.0e30; }
int EVTdequeue(void) { return 0; }
int EVTbackup(void) { return 0; }
int EVTaccept(void) { return 0; }
int EVTsetup(void) { return 0; }
int EVTdest(void) { return 0; }
int MIF_INP2A(void) { return 0; }
int CKTsoaInit(void) { return 0; }
int CKTsoaCheck(void) { return 0; }
int INPgetTree(void) { return 1; }
void INPptPrint(void) { }
/* Transient-noise and random sources (TRNOISE/TRRANDOM waveforms) are not
 * used by the oracle netlists. */
void *trnoise_state_init(void) { return 0; }
void trnoise_state_free(void) { }
int trnoise_state_gen(void) { return 0; }
void *trrandom_state_init(void) { return 0; }
double gauss0(void) { return 0.0; }
double exprand(void) { return 0.0; }
double drand(void) { return 0.0; }
int poisson(void) { return 0; }
void fftFree(void) { }
void *slogp = 0;
