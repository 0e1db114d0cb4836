// C++-linkage aliases of the task runtime and the spe* wrappers.
//
// The reference declares celldsp_* (cellspe-tasklib.h:122-133) and the spe*
// wrappers (cellspe-tasklib-dsp.h:79-94) without extern "C", so a caller
// compiled against those headers links against the C++-mangled names
// (_Z13celldsp_startv, _Z17celldsp_startTaskiP14CellDSPTask_tt,
// _Z18speAddProduct_32fcP4fc32S0_S0_i, ...).  This file exports those names
// as well; each forwards to the extern "C" entry point of the same name, so
// an already-built C++ caller links unchanged, and callers compiled against
// include/cellspe-tasklib*.h use the C names.
//
// The mangled names depend on the parameter types' names, so the types are
// declared here exactly as the reference names them: the task descriptor's
// struct tag CellDSPTask_tt and fc32 as a typedef of an unnamed struct
// (types_generic.h:44-45; cf32 is the same type).  This file does not include
// the engine's headers: their extern "C" declarations of the same names
// would clash with the C++ definitions below.  The C symbols are reached
// through asm labels on differently named declarations.
struct CellDSPTask_tt;
typedef CellDSPTask_tt CellDSPTask_t;
typedef struct {
    float re;
    float im;
} fc32;
typedef fc32 cf32;

#define CS_C_SYMBOL(name) __asm__(#name)

extern "C" {
int cs_c_start(void) CS_C_SYMBOL(celldsp_start);
int cs_c_stop(void) CS_C_SYMBOL(celldsp_stop);
int cs_c_getFreeSPE(void) CS_C_SYMBOL(celldsp_getFreeSPE);
int cs_c_setFreeSPE(int) CS_C_SYMBOL(celldsp_setFreeSPE);
int cs_c_startTask(int, CellDSPTask_t*) CS_C_SYMBOL(celldsp_startTask);
int cs_c_waitTask(int) CS_C_SYMBOL(celldsp_waitTask);
int cs_c_executeTask(CellDSPTask_t*) CS_C_SYMBOL(celldsp_executeTask);
int cs_c_startContinuableTask(CellDSPTask_t*, int*) CS_C_SYMBOL(celldsp_startContinuableTask);
int cs_c_continueTask(CellDSPTask_t*, int*) CS_C_SYMBOL(celldsp_continueTask);
int cs_c_stopContinuableTask(int*) CS_C_SYMBOL(celldsp_stopContinuableTask);
void cs_c_setBehaviour(unsigned int) CS_C_SYMBOL(celldsp_setBehaviour);
unsigned int cs_c_getBehaviour(void) CS_C_SYMBOL(celldsp_getBehaviour);

int cs_c_speNOP(void) CS_C_SYMBOL(speNOP);
int cs_c_speRunAllCheck(void) CS_C_SYMBOL(speRunAllCheck);
int cs_c_speIOCheck(void) CS_C_SYMBOL(speIOCheck);
int cs_c_speIOSimulation(void) CS_C_SYMBOL(speIOSimulation);
int cs_c_speIOBench(void*, unsigned int, int) CS_C_SYMBOL(speIOBench);
int cs_c_speIOBenchStreamed(void*, unsigned int, int, int) CS_C_SYMBOL(speIOBenchStreamed);
int cs_c_speAddProduct_32fc(fc32*, fc32*, fc32*, int) CS_C_SYMBOL(speAddProduct_32fc);
int cs_c_speFFT_init(int, int*) CS_C_SYMBOL(speFFT_init);
int cs_c_speFFT_exec(void*, void*, int, int*) CS_C_SYMBOL(speFFT_exec);
int cs_c_speFFT_destroy(int*) CS_C_SYMBOL(speFFT_destroy);
int cs_c_speFFT_singleexec(void*, void*, int) CS_C_SYMBOL(speFFT_singleexec);
int cs_c_speDIFX_process(void*, void*, void*, void*, void*, int, int, int) CS_C_SYMBOL(speDIFX_process);
int cs_c_speSinCosGenerator(float, float, fc32*, int) CS_C_SYMBOL(speSinCosGenerator);
int cs_c_speSinCosAccurate(float*, cf32*, int) CS_C_SYMBOL(speSinCosAccurate);
int cs_c_speSinCosAccurateNorm(float*, cf32*, int) CS_C_SYMBOL(speSinCosAccurateNorm);
}

// cellspe-tasklib.h:122-133
int celldsp_start() { return cs_c_start(); }
int celldsp_stop() { return cs_c_stop(); }
int celldsp_getFreeSPE() { return cs_c_getFreeSPE(); }
int celldsp_setFreeSPE(int targetSPE) { return cs_c_setFreeSPE(targetSPE); }
int celldsp_startTask(int targetSPE, CellDSPTask_t* task) { return cs_c_startTask(targetSPE, task); }
int celldsp_waitTask(int targetSPE) { return cs_c_waitTask(targetSPE); }
int celldsp_executeTask(CellDSPTask_t* task) { return cs_c_executeTask(task); }
int celldsp_startContinuableTask(CellDSPTask_t* task, int* speID) { return cs_c_startContinuableTask(task, speID); }
int celldsp_continueTask(CellDSPTask_t* task, int* speID) { return cs_c_continueTask(task, speID); }
int celldsp_stopContinuableTask(int* speID) { return cs_c_stopContinuableTask(speID); }
void celldsp_setBehaviour(unsigned int flags) { cs_c_setBehaviour(flags); }
unsigned int celldsp_getBehaviour() { return cs_c_getBehaviour(); }

// cellspe-tasklib-dsp.h:79-94
int speNOP() { return cs_c_speNOP(); }
int speRunAllCheck() { return cs_c_speRunAllCheck(); }
int speIOCheck() { return cs_c_speIOCheck(); }
int speIOSimulation() { return cs_c_speIOSimulation(); }
int speIOBench(void* buffer, unsigned int bufbytes, int spes) { return cs_c_speIOBench(buffer, bufbytes, spes); }
int speIOBenchStreamed(void* buffer, unsigned int bufbytes, int spes, int stream_length)
{
    return cs_c_speIOBenchStreamed(buffer, bufbytes, spes, stream_length);
}
int speAddProduct_32fc(fc32* src, fc32* src2, fc32* accumulator, int length)
{
    return cs_c_speAddProduct_32fc(src, src2, accumulator, length);
}
int speFFT_init(int fft_len, int* speID) { return cs_c_speFFT_init(fft_len, speID); }
int speFFT_exec(void* in, void* out, int fft_len, int* speID) { return cs_c_speFFT_exec(in, out, fft_len, speID); }
int speFFT_destroy(int* speID) { return cs_c_speFFT_destroy(speID); }
int speFFT_singleexec(void* in, void* out, int fft_len) { return cs_c_speFFT_singleexec(in, out, fft_len); }
int speDIFX_process(void* sincosrotdone, void* complexfracmult, void* fftoutJ, void* conjfftoutJ, void* autocorr,
                    int nfft, int twicenumchannels, int useUpperOrLower)
{
    return cs_c_speDIFX_process(sincosrotdone, complexfracmult, fftoutJ, conjfftoutJ, autocorr, nfft,
                                twicenumchannels, useUpperOrLower);
}
int speSinCosGenerator(float startphase, float increment, fc32* cos_sin_out, int numiter)
{
    return cs_c_speSinCosGenerator(startphase, increment, cos_sin_out, numiter);
}
int speSinCosAccurate(float* argument, cf32* cos_sin_out, int argumentcount)
{
    return cs_c_speSinCosAccurate(argument, cos_sin_out, argumentcount);
}
int speSinCosAccurateNorm(float* normalizedargument, cf32* cos_sin_out, int argumentcount)
{
    return cs_c_speSinCosAccurateNorm(normalizedargument, cos_sin_out, argumentcount);
}
