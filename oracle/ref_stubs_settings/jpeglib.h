/* Stand-in for <jpeglib.h>: src/files.h embeds a jpeg_error_mgr and names JSAMPLE in
 * declarations the settings harness never calls. Test infrastructure only. */
#ifndef MBGB_REF_STUB_JPEGLIB_H
#define MBGB_REF_STUB_JPEGLIB_H
typedef unsigned char JSAMPLE;
struct jpeg_error_mgr { int unused; };
#endif
