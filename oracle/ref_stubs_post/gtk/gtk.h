/* Stand-in for <gtk/gtk.h> used only to compile the reference's image post-processing
 * sources (src/image.cpp, src/cimage.cpp) for the oracle's pinning harness. It carries
 * the typedefs of the hot-path stub plus no-op definitions of the GTK/GDK/GLib calls
 * those files make on their GUI paths (progress bars, previews, drawing), which the
 * harness never reaches: it runs with noGUI set. g_thread_create runs the thread body
 * synchronously. Test infrastructure only. */
#ifndef MBGB_REF_STUB_GTK_POST_H
#define MBGB_REF_STUB_GTK_POST_H
#include <time.h>
typedef unsigned long long guint64;
typedef int gboolean;
typedef int gint;
typedef unsigned int guint;
typedef double gdouble;
typedef unsigned char guchar;
typedef void *gpointer;
typedef char gchar;
#define TRUE 1
#define FALSE 0
struct GdkGC;
typedef struct GdkGC GdkGC;
struct GdkDrawable;
struct GtkStyle { GdkGC *fg_gc[5]; };
struct GtkWidget { struct GdkDrawable *window; struct GtkStyle *style; };
struct GtkWindow; struct GtkObject; struct GtkAdjustment; struct GtkClipboard;
struct GtkSelectionData; struct GtkFileChooser; struct GtkTreeView; struct GtkListStore; struct GtkTreeIter;
struct GtkTextBuffer; struct GtkComboBox; struct GtkProgressBar;
struct GdkEventMotion; struct GdkEventButton; struct GdkEvent; struct GdkEventExpose; struct GdkEventKey;
struct GdkEventConfigure; struct GdkEventScroll; struct GdkDragContext;
struct GdkColor { unsigned int pixel; unsigned short red, green, blue; };
typedef struct { int unused; } GThread;
typedef struct { int unused; } GError;
typedef void *(*GThreadFunc)(void *);
#define GTK_STATE_NORMAL 0
#define GDK_RGB_DITHER_MAX 0
#define GTK_PROGRESS_BAR(x) (x)
#define GTK_ADJUSTMENT(x) (x)
static inline void gtk_progress_bar_set_text(void *, const char *) {}
static inline gboolean gtk_events_pending(void) { return 0; }
static inline void gtk_main_iteration(void) {}
static inline double gtk_adjustment_get_value(void *) { return 0.0; }
static inline void gdk_draw_rgb_image(void *, void *, int, int, int, int, int, const void *, int) {}
static inline void gdk_draw_rectangle(void *, void *, int, int, int, int, int) {}
static inline void gdk_draw_line(void *, void *, int, int, int, int) {}
static inline GdkGC *gdk_gc_new(void *) { return 0; }
static inline void gdk_gc_set_rgb_fg_color(void *, const GdkColor *) {}
static inline GThread *g_thread_create(GThreadFunc f, void *arg, gboolean, GError **) {
  static GThread t;
  f(arg);
  return &t;
}
static inline void *g_thread_join(GThread *) { return 0; }
#ifndef MAX
#define MAX(a, b) (((a) > (b)) ? (a) : (b))
#endif
#ifndef MIN
#define MIN(a, b) (((a) < (b)) ? (a) : (b))
#endif
#endif
