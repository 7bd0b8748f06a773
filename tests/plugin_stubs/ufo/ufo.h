/*
 * Declarations of the glib / GObject / ufo-core API that the plugin shells
 * (the .c files under plugins/) use, for a compile check where those libraries are absent.
 * Test infrastructure: nothing here is linked or run. Types and signatures
 * follow the public glib 2.x and ufo-core headers; macros that generate code
 * (G_DEFINE_TYPE_WITH_CODE, G_IMPLEMENT_INTERFACE) expand to the functions
 * and statics the real ones define that the shells refer to.
 */
#ifndef PLUGIN_STUBS_UFO_H
#define PLUGIN_STUBS_UFO_H

#include <float.h>
#include <limits.h>
#include <stddef.h>

#define G_BEGIN_DECLS
#define G_END_DECLS
#define TRUE 1
#define FALSE 0
#define G_MAXUINT UINT_MAX
#define G_MAXFLOAT FLT_MAX
#define G_MINFLOAT FLT_MIN

typedef int gboolean;
typedef int gint;
typedef unsigned int guint;
typedef float gfloat;
typedef char gchar;
typedef void *gpointer;
typedef size_t GType;
typedef unsigned int GQuark;

typedef struct _GValue { GType g_type; double data[2]; } GValue;
typedef struct _GParamSpec GParamSpec;
typedef struct _GError { GQuark domain; gint code; gchar *message; } GError;
typedef struct _GMutex { gpointer p; guint i[2]; } GMutex;
typedef enum { G_PARAM_READABLE = 1 << 0, G_PARAM_WRITABLE = 1 << 1, G_PARAM_READWRITE = 3 } GParamFlags;

typedef struct _GTypeInstance { gpointer g_class; } GTypeInstance;
typedef struct _GObject { GTypeInstance g_type_instance; guint ref_count; gpointer qdata; } GObject;
typedef struct _GObjectClass {
    gpointer g_type_class;
    gpointer construct_properties;
    GObject *(*constructor) (GType, guint, gpointer);
    void (*set_property) (GObject *object, guint property_id, const GValue *value, GParamSpec *pspec);
    void (*get_property) (GObject *object, guint property_id, GValue *value, GParamSpec *pspec);
    void (*dispose) (GObject *object);
    void (*finalize) (GObject *object);
    gpointer pdummy[8];
} GObjectClass;
typedef void (*GClassInitFunc) (gpointer g_class, gpointer class_data);
typedef void (*GInstanceInitFunc) (GTypeInstance *instance, gpointer g_class);
typedef void (*GInterfaceInitFunc) (gpointer g_iface, gpointer iface_data);
typedef struct { GInterfaceInitFunc interface_init; gpointer interface_finalize; gpointer interface_data; } GInterfaceInfo;

GType g_object_get_type (void);
#define G_TYPE_OBJECT (g_object_get_type ())
#define G_OBJECT(obj) ((GObject *) (obj))
#define G_OBJECT_CLASS(klass) ((GObjectClass *) (klass))
#define G_OBJECT_WARN_INVALID_PROPERTY_ID(object, property_id, pspec) \
    g_warning ("invalid property id %u", (guint) (property_id))
#define g_return_val_if_fail(expr, val) do { if (!(expr)) return (val); } while (0)

GType g_type_register_static_simple (GType parent, const gchar *name, guint class_size, GClassInitFunc class_init,
                                     guint instance_size, GInstanceInitFunc instance_init, gint flags);
void g_type_add_interface_static (GType instance_type, GType interface_type, const GInterfaceInfo *info);
gpointer g_type_class_peek_parent (gpointer g_class);

#define G_DEFINE_TYPE_WITH_CODE(TN, t_n, T_P, _C_)                                                        \
    static void t_n##_init (TN *self);                                                                     \
    static void t_n##_class_init (TN##Class *klass);                                                       \
    static gpointer t_n##_parent_class = NULL;                                                             \
    static void t_n##_class_intern_init (gpointer klass, gpointer data)                                    \
    {                                                                                                      \
        (void) data;                                                                                       \
        t_n##_parent_class = g_type_class_peek_parent (klass);                                             \
        t_n##_class_init ((TN##Class *) klass);                                                            \
    }                                                                                                      \
    static void t_n##_instance_init (GTypeInstance *inst, gpointer klass)                                  \
    {                                                                                                      \
        (void) klass;                                                                                      \
        t_n##_init ((TN *) inst);                                                                          \
    }                                                                                                      \
    GType t_n##_get_type (void);                                                                           \
    GType t_n##_get_type (void)                                                                            \
    {                                                                                                      \
        static GType g_define_type_id = 0;                                                                 \
        if (g_define_type_id == 0) {                                                                       \
            g_define_type_id = g_type_register_static_simple (T_P, #TN, sizeof (TN##Class),                \
                                                              t_n##_class_intern_init, sizeof (TN),        \
                                                              t_n##_instance_init, 0);                     \
            { _C_; }                                                                                       \
        }                                                                                                  \
        return g_define_type_id;                                                                           \
    }
#define G_IMPLEMENT_INTERFACE(TYPE_IFACE, iface_init)                                                     \
    {                                                                                                      \
        const GInterfaceInfo g_implement_interface_info = {(GInterfaceInitFunc) (void (*) (void)) iface_init, \
                                                           NULL, NULL};                                    \
        g_type_add_interface_static (g_define_type_id, TYPE_IFACE, &g_implement_interface_info);           \
    }

gpointer g_object_new (GType object_type, const gchar *first_property_name, ...);
gpointer g_object_ref (gpointer object);
gpointer g_object_ref_sink (gpointer object);
void g_object_unref (gpointer object);
void g_object_get (gpointer object, const gchar *first_property_name, ...);
void g_object_set_data (GObject *object, const gchar *key, gpointer data);
gpointer g_object_get_data (GObject *object, const gchar *key);
void g_object_class_install_property (GObjectClass *oclass, guint property_id, GParamSpec *pspec);
GParamSpec *g_param_spec_uint (const gchar *name, const gchar *nick, const gchar *blurb, guint minimum,
                               guint maximum, guint default_value, GParamFlags flags);
GParamSpec *g_param_spec_float (const gchar *name, const gchar *nick, const gchar *blurb, gfloat minimum,
                                gfloat maximum, gfloat default_value, GParamFlags flags);
GParamSpec *g_param_spec_boolean (const gchar *name, const gchar *nick, const gchar *blurb,
                                  gboolean default_value, GParamFlags flags);
GParamSpec *g_param_spec_string (const gchar *name, const gchar *nick, const gchar *blurb,
                                 const gchar *default_value, GParamFlags flags);
GParamSpec *g_param_spec_object (const gchar *name, const gchar *nick, const gchar *blurb, GType object_type,
                                 GParamFlags flags);
guint g_value_get_uint (const GValue *value);
gfloat g_value_get_float (const GValue *value);
gboolean g_value_get_boolean (const GValue *value);
const gchar *g_value_get_string (const GValue *value);
gchar *g_value_dup_string (const GValue *value);
gpointer g_value_get_object (const GValue *value);
void g_value_set_uint (GValue *value, guint v);
void g_value_set_float (GValue *value, gfloat v);
void g_value_set_boolean (GValue *value, gboolean v);
void g_value_set_string (GValue *value, const gchar *v);
void g_value_set_object (GValue *value, gpointer v);
void g_set_error (GError **err, GQuark domain, gint code, const gchar *format, ...)
    __attribute__ ((format (printf, 4, 5)));
void g_warning (const gchar *format, ...) __attribute__ ((format (printf, 1, 2)));
const gchar *g_getenv (const gchar *variable);
void g_mutex_lock (GMutex *mutex);
void g_mutex_unlock (GMutex *mutex);
size_t g_strlcpy (gchar *dest, const gchar *src, size_t dest_size);
gchar *g_strdup (const gchar *str);
void g_free (gpointer mem);
gint g_ascii_strcasecmp (const gchar *s1, const gchar *s2);

/* ufo-core */
typedef struct _UfoNode { GObject parent_instance; gpointer priv; } UfoNode;
typedef struct _UfoTaskNode { UfoNode parent_instance; gpointer priv; } UfoTaskNode;
typedef struct _UfoTaskNodeClass { GObjectClass parent_class; gpointer node_class[4]; } UfoTaskNodeClass;
typedef struct _UfoTask UfoTask;
typedef struct _UfoResources UfoResources;
typedef struct _UfoBuffer UfoBuffer;
#define UFO_BUFFER_MAX_NDIMS 3
typedef struct _UfoRequisition { guint n_dims; size_t dims[UFO_BUFFER_MAX_NDIMS]; } UfoRequisition;
typedef enum {
    UFO_TASK_MODE_INVALID = 0,
    UFO_TASK_MODE_PROCESSOR = 1 << 0,
    UFO_TASK_MODE_GENERATOR = 1 << 1,
    UFO_TASK_MODE_REDUCTOR = 1 << 2,
    UFO_TASK_MODE_CPU = 1 << 3,
    UFO_TASK_MODE_GPU = 1 << 4
} UfoTaskMode;
typedef struct _UfoTaskIface {
    gpointer parent_iface[2];
    void (*setup) (UfoTask *task, UfoResources *resources, GError **error);
    void (*get_requisition) (UfoTask *task, UfoBuffer **inputs, UfoRequisition *requisition, GError **error);
    guint (*get_num_inputs) (UfoTask *task);
    guint (*get_num_dimensions) (UfoTask *task, guint input);
    UfoTaskMode (*get_mode) (UfoTask *task);
    gboolean (*set_json_object_property) (UfoTask *task, const gchar *prop_name, gpointer object);
    gboolean (*process) (UfoTask *task, UfoBuffer **inputs, UfoBuffer *output, UfoRequisition *requisition);
    gboolean (*generate) (UfoTask *task, UfoBuffer *output, UfoRequisition *requisition);
} UfoTaskIface;
typedef enum { UFO_TASK_ERROR_SETUP } UfoTaskError;
GQuark ufo_task_error_quark (void);
#define UFO_TASK_ERROR (ufo_task_error_quark ())
GType ufo_task_node_get_type (void);
GType ufo_task_get_type (void);
#define UFO_TYPE_TASK_NODE (ufo_task_node_get_type ())
#define UFO_TYPE_TASK (ufo_task_get_type ())
#define UFO_NODE(obj) ((UfoNode *) (obj))
#define UFO_TASK(obj) ((UfoTask *) (obj))
void ufo_task_setup (UfoTask *task, UfoResources *resources, GError **error);
void ufo_buffer_get_requisition (UfoBuffer *buffer, UfoRequisition *requisition);
gfloat *ufo_buffer_get_host_array (UfoBuffer *buffer, gpointer cmd_queue);

#endif
