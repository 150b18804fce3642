/* Minimal stand-in for <gtk/gtk.h>, only so the reference's hot-path sources
 * (fractal.cpp, shaders.cpp, algebra.cpp, common_math.cpp, primitives.cpp)
 * compile without GTK: the basic GLib typedefs, opaque widget/event types that
 * the included headers name in declarations, GdkColor and the MAX/MIN macros.
 * Nothing here is called at run time. Test infrastructure only. */
#ifndef MBGB_REF_STUB_GTK_H
#define MBGB_REF_STUB_GTK_H
typedef unsigned long long guint64;
typedef int gboolean;
typedef int gint;
typedef unsigned int guint;
typedef double gdouble;
typedef unsigned char guchar;
typedef void *gpointer;
typedef char gchar;
struct GtkWidget; struct GtkWindow; struct GtkObject; struct GtkAdjustment; struct GtkClipboard;
struct GtkSelectionData; struct GtkFileChooser; struct GtkTreeView; struct GtkListStore; struct GtkTreeIter;
struct GtkTextBuffer; struct GtkComboBox;
struct GdkEventMotion; struct GdkEventButton; struct GdkEvent; struct GdkEventExpose; struct GdkEventKey;
struct GdkEventConfigure; struct GdkEventScroll; struct GdkDragContext;
struct GdkColor { unsigned int pixel; unsigned short red, green, blue; };
#ifndef MAX
#define MAX(a, b) (((a) > (b)) ? (a) : (b))
#endif
#ifndef MIN
#define MIN(a, b) (((a) < (b)) ? (a) : (b))
#endif
#endif
