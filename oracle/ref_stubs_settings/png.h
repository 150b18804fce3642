/* Stand-in for <png.h>: the reference's src/files.h names png_byte in declarations of
 * functions the settings harness never calls. Test infrastructure only. */
#ifndef MBGB_REF_STUB_PNG_H
#define MBGB_REF_STUB_PNG_H
typedef unsigned char png_byte;
#endif
