/* NVTX injection library for tests/test_trace.py: the NVTX v3 headers that libsvo includes load the
 * library named by NVTX_INJECTION64_PATH at the first NVTX call and hand it the core callback table;
 * this probe appends "push <name>" and "pop" lines to the file named by NVTX_PROBE_OUT. */
#include <stdio.h>
#include <stdlib.h>

#include <nvtx3/nvToolsExt.h>

static FILE* out;

static int probe_push(const char* message) {
  if (out) {
    fprintf(out, "push %s\n", message ? message : "");
    fflush(out);
  }
  return 0;
}

static int probe_pop(void) {
  if (out) {
    fputs("pop\n", out);
    fflush(out);
  }
  return 0;
}

int InitializeInjectionNvtx2(NvtxGetExportTableFunc_t get_export_table) {
  const NvtxExportTableCallbacks* cb = (const NvtxExportTableCallbacks*)get_export_table(NVTX_ETID_CALLBACKS);
  NvtxFunctionTable table = 0;
  unsigned int size = 0;
  if (!cb || !cb->GetModuleFunctionTable(NVTX_CB_MODULE_CORE, &table, &size) || size <= NVTX_CBID_CORE_RangePop)
    return 0;
  *table[NVTX_CBID_CORE_RangePushA] = (NvtxFunctionPointer)probe_push;
  *table[NVTX_CBID_CORE_RangePop] = (NvtxFunctionPointer)probe_pop;
  const char* path = getenv("NVTX_PROBE_OUT");
  out = path ? fopen(path, "w") : NULL;
  return 1;
}
