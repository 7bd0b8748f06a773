/*
 * ufo-ir-sbtv-task.c - the "sbtv" node of package "ir" over libufoir.
 *
 * Replaces src/tasks/ufo-ir-sbtv-task.c: properties lambda ([0, MAX], 0.1)
 * and mu ([0, MAX], 0.5) (:90-101) on top of the method base; process
 * (:230-302) is ufoir_sbtv_process. The reference normalises its input
 * sinogram in place (:239); libufoir works on a normalised copy and leaves
 * the input buffer as it was. Extension: "norm-mode" ("fp64", the default,
 * or "compat": the reference's float sequential sums).
 */
#include "ufo-ir-method-shell.h"

typedef struct {
    UfoIrMethodShell base;
    gfloat lambda, mu;
    gchar *norm_mode;
} UfoIrSbtvTask;

typedef struct {
    UfoTaskNodeClass parent_class;
} UfoIrSbtvTaskClass;

static void ufo_task_interface_init (UfoTaskIface *iface);

G_DEFINE_TYPE_WITH_CODE (UfoIrSbtvTask, ufo_ir_sbtv_task, UFO_TYPE_TASK_NODE,
                         G_IMPLEMENT_INTERFACE (UFO_TYPE_TASK, ufo_task_interface_init))

#define SELF(obj) ((UfoIrSbtvTask *) (obj))

enum { PROP_LAMBDA = UFO_IR_METHOD_PROP_FIRST_OWN, PROP_MU, PROP_NORM_MODE };

UfoNode *
ufo_ir_sbtv_task_new (void)
{
    return UFO_NODE (g_object_new (ufo_ir_sbtv_task_get_type (), NULL));
}

static void
ufo_ir_sbtv_task_set_property (GObject *object, guint property_id, const GValue *value, GParamSpec *pspec)
{
    UfoIrSbtvTask *self = SELF (object);

    if (ufo_ir_method_shell_set (&self->base, property_id, value))
        return;
    switch (property_id) {
        case PROP_LAMBDA: self->lambda = g_value_get_float (value); break;
        case PROP_MU: self->mu = g_value_get_float (value); break;
        case PROP_NORM_MODE:
            g_free (self->norm_mode);
            self->norm_mode = g_value_dup_string (value);
            break;
        default:
            G_OBJECT_WARN_INVALID_PROPERTY_ID (object, property_id, pspec);
            break;
    }
}

static void
ufo_ir_sbtv_task_get_property (GObject *object, guint property_id, GValue *value, GParamSpec *pspec)
{
    UfoIrSbtvTask *self = SELF (object);

    if (ufo_ir_method_shell_get (&self->base, property_id, value))
        return;
    switch (property_id) {
        case PROP_LAMBDA: g_value_set_float (value, self->lambda); break;
        case PROP_MU: g_value_set_float (value, self->mu); break;
        case PROP_NORM_MODE: g_value_set_string (value, self->norm_mode); break;
        default:
            G_OBJECT_WARN_INVALID_PROPERTY_ID (object, property_id, pspec);
            break;
    }
}

static void
ufo_ir_sbtv_task_dispose (GObject *object)
{
    ufo_ir_method_shell_dispose (&SELF (object)->base);
    G_OBJECT_CLASS (ufo_ir_sbtv_task_parent_class)->dispose (object);
}

static void
ufo_ir_sbtv_task_finalize (GObject *object)
{
    g_free (SELF (object)->norm_mode);
    G_OBJECT_CLASS (ufo_ir_sbtv_task_parent_class)->finalize (object);
}

static void
ufo_ir_sbtv_task_setup (UfoTask *task, UfoResources *resources, GError **error)
{
    ufo_ir_method_shell_setup (&SELF (task)->base, resources, error);
}

static void
ufo_ir_sbtv_task_get_requisition (UfoTask *task, UfoBuffer **inputs, UfoRequisition *requisition, GError **error)
{
    ufo_ir_shell_method_requisition (SELF (task)->base.projector, inputs, requisition, error);
}

static guint
ufo_ir_sbtv_task_get_num_inputs (UfoTask *task)
{
    return 1;
}

static guint
ufo_ir_sbtv_task_get_num_dimensions (UfoTask *task, guint input)
{
    g_return_val_if_fail (input == 0, 0);
    return 2;
}

static UfoTaskMode
ufo_ir_sbtv_task_get_mode (UfoTask *task)
{
    return UFO_TASK_MODE_PROCESSOR | UFO_TASK_MODE_CPU;
}

static gboolean
ufo_ir_sbtv_task_process (UfoTask *task, UfoBuffer **inputs, UfoBuffer *output, UfoRequisition *requisition)
{
    UfoIrSbtvTask *self = SELF (task);
    ufoir_projector *proj = ufo_ir_shell_projector (self->base.projector, NULL);
    ufoir_sbtv_params prm;
    size_t dims[2];

    if (proj == NULL)
        return ufo_ir_method_shell_done ("sbtv", UFOIR_ERR_STATE);
    ufoir_sbtv_params_init (&prm);
    prm.num_iterations = self->base.num_iterations;
    prm.lambda = self->lambda;
    prm.mu = self->mu;
    prm.norm_mode = ufo_ir_shell_norm_mode (self->norm_mode);
    ufo_ir_method_shell_dims (inputs[0], dims);
    return ufo_ir_method_shell_done ("sbtv",
        ufoir_sbtv_process (proj, &prm, ufo_buffer_get_host_array (inputs[0], NULL), dims,
                            ufo_buffer_get_host_array (output, NULL), 1));
}

static void
ufo_task_interface_init (UfoTaskIface *iface)
{
    iface->setup = ufo_ir_sbtv_task_setup;
    iface->get_requisition = ufo_ir_sbtv_task_get_requisition;
    iface->get_num_inputs = ufo_ir_sbtv_task_get_num_inputs;
    iface->get_num_dimensions = ufo_ir_sbtv_task_get_num_dimensions;
    iface->get_mode = ufo_ir_sbtv_task_get_mode;
    iface->process = ufo_ir_sbtv_task_process;
}

static void
ufo_ir_sbtv_task_class_init (UfoIrSbtvTaskClass *klass)
{
    GObjectClass *oclass = G_OBJECT_CLASS (klass);

    oclass->set_property = ufo_ir_sbtv_task_set_property;
    oclass->get_property = ufo_ir_sbtv_task_get_property;
    oclass->dispose = ufo_ir_sbtv_task_dispose;
    oclass->finalize = ufo_ir_sbtv_task_finalize;
    ufo_ir_method_shell_install (oclass);
    g_object_class_install_property (oclass, PROP_LAMBDA,
        g_param_spec_float ("lambda", "Lambda", "Lambda", 0.0f, G_MAXFLOAT, 0.1f, G_PARAM_READWRITE));
    g_object_class_install_property (oclass, PROP_MU,
        g_param_spec_float ("mu", "Mu", "Mu", 0.0f, G_MAXFLOAT, 0.5f, G_PARAM_READWRITE));
    g_object_class_install_property (oclass, PROP_NORM_MODE,
        g_param_spec_string ("norm-mode", "Norm arithmetic", "fp64 (default) or compat", "fp64",
                             G_PARAM_READWRITE));
}

static void
ufo_ir_sbtv_task_init (UfoIrSbtvTask *self)
{
    ufo_ir_method_shell_init (&self->base);
    self->lambda = 0.1f;
    self->mu = 0.5f;
    self->norm_mode = g_strdup ("fp64");
}
