// Embeds the table written by gen_libm_expf (arguments where this machine's
// C library expf is not the correctly rounded value) into the library.
// SWE_LIBM_EXPF_BIN is the absolute path of that file, set by the build.
#define SWE_STR2(x) #x
#define SWE_STR(x) SWE_STR2(x)

__asm__(
    ".section .rodata\n"
    ".balign 16\n"
    ".global swe_libm_expf_blob\n"
    ".hidden swe_libm_expf_blob\n"
    "swe_libm_expf_blob:\n"
    ".incbin \"" SWE_STR(SWE_LIBM_EXPF_BIN) "\"\n"
    ".global swe_libm_expf_blob_end\n"
    ".hidden swe_libm_expf_blob_end\n"
    "swe_libm_expf_blob_end:\n"
    ".byte 0\n"
    ".previous\n");
