/*
 * ufo-ir-asdpocs-task.c - the "asdpocs" node of package "ir" over libufoir.
 *
 * Replaces src/tasks/ufo-ir-asdpocs-task.c: properties beta, beta_red,
 * alpha, alpha_red, r_max ([0, MAX], defaults 1, 0.995, 0.2, 0.95, 0.95),
 * ng ([0, 1000], 20, accepted and unused as in the reference, which
 * hard-codes 20 TV sub-steps at :573), positive_constraint (TRUE) and
 * df_minimizer (a "sart" node whose num-iterations and relaxation_factor
 * the inner SART uses) (:104-181), on top of the method base; process
 * (:411-509) is ufoir_asdpocs_process. Extension: "norm-mode" ("fp64",
 * the default, or "compat": the reference's float sequential sums).
 */
#include "ufo-ir-method-shell.h"

typedef struct {
    UfoIrMethodShell base;
    gfloat beta, beta_red, alpha, alpha_red, r_max;
    guint ng;
    gboolean positive_constraint;
    GObject *df_minimizer;
    gchar *norm_mode;
} UfoIrAsdpocsTask;

typedef struct {
    UfoTaskNodeClass parent_class;
} UfoIrAsdpocsTaskClass;

static void ufo_task_interface_init (UfoTaskIface *iface);

G_DEFINE_TYPE_WITH_CODE (UfoIrAsdpocsTask, ufo_ir_asdpocs_task, UFO_TYPE_TASK_NODE,
                         G_IMPLEMENT_INTERFACE (UFO_TYPE_TASK, ufo_task_interface_init))

#define SELF(obj) ((UfoIrAsdpocsTask *) (obj))

enum {
    PROP_BETA = UFO_IR_METHOD_PROP_FIRST_OWN,
    PROP_BETA_RED,
    PROP_NG,
    PROP_ALPHA,
    PROP_ALPHA_RED,
    PROP_R_MAX,
    PROP_POSITIVE_CONSTRAINT,
    PROP_DF_MINIMIZER,
    PROP_NORM_MODE
};

UfoNode *
ufo_ir_asdpocs_task_new (void)
{
    return UFO_NODE (g_object_new (ufo_ir_asdpocs_task_get_type (), NULL));
}

static void
ufo_ir_asdpocs_task_set_property (GObject *object, guint property_id, const GValue *value, GParamSpec *pspec)
{
    UfoIrAsdpocsTask *self = SELF (object);

    if (ufo_ir_method_shell_set (&self->base, property_id, value))
        return;
    switch (property_id) {
        case PROP_BETA: self->beta = g_value_get_float (value); break;
        case PROP_BETA_RED: self->beta_red = g_value_get_float (value); break;
        case PROP_NG: self->ng = g_value_get_uint (value); break;
        case PROP_ALPHA: self->alpha = g_value_get_float (value); break;
        case PROP_ALPHA_RED: self->alpha_red = g_value_get_float (value); break;
        case PROP_R_MAX: self->r_max = g_value_get_float (value); break;
        case PROP_POSITIVE_CONSTRAINT: self->positive_constraint = g_value_get_boolean (value); break;
        case PROP_DF_MINIMIZER: {
            GObject *m = g_value_get_object (value);
            if (self->df_minimizer != NULL)
                g_object_unref (self->df_minimizer);
            self->df_minimizer = m != NULL ? g_object_ref (m) : NULL;
            break;
        }
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
ufo_ir_asdpocs_task_get_property (GObject *object, guint property_id, GValue *value, GParamSpec *pspec)
{
    UfoIrAsdpocsTask *self = SELF (object);

    if (ufo_ir_method_shell_get (&self->base, property_id, value))
        return;
    switch (property_id) {
        case PROP_BETA: g_value_set_float (value, self->beta); break;
        case PROP_BETA_RED: g_value_set_float (value, self->beta_red); break;
        case PROP_NG: g_value_set_uint (value, self->ng); break;
        case PROP_ALPHA: g_value_set_float (value, self->alpha); break;
        case PROP_ALPHA_RED: g_value_set_float (value, self->alpha_red); break;
        case PROP_R_MAX: g_value_set_float (value, self->r_max); break;
        case PROP_POSITIVE_CONSTRAINT: g_value_set_boolean (value, self->positive_constraint); break;
        case PROP_DF_MINIMIZER: g_value_set_object (value, self->df_minimizer); break;
        case PROP_NORM_MODE: g_value_set_string (value, self->norm_mode); break;
        default:
            G_OBJECT_WARN_INVALID_PROPERTY_ID (object, property_id, pspec);
            break;
    }
}

static void
ufo_ir_asdpocs_task_dispose (GObject *object)
{
    UfoIrAsdpocsTask *self = SELF (object);

    ufo_ir_method_shell_dispose (&self->base);
    if (self->df_minimizer != NULL) {
        g_object_unref (self->df_minimizer);
        self->df_minimizer = NULL;
    }
    G_OBJECT_CLASS (ufo_ir_asdpocs_task_parent_class)->dispose (object);
}

static void
ufo_ir_asdpocs_task_finalize (GObject *object)
{
    g_free (SELF (object)->norm_mode);
    G_OBJECT_CLASS (ufo_ir_asdpocs_task_parent_class)->finalize (object);
}

static void
ufo_ir_asdpocs_task_setup (UfoTask *task, UfoResources *resources, GError **error)
{
    UfoIrAsdpocsTask *self = SELF (task);

    /* the reference requires a minimizer (:282-290) */
    if (self->df_minimizer == NULL) {
        g_set_error (error, UFO_TASK_ERROR, UFO_TASK_ERROR_SETUP, "No df_minimizer specified.");
        return;
    }
    ufo_ir_method_shell_setup (&self->base, resources, error);
}

static void
ufo_ir_asdpocs_task_get_requisition (UfoTask *task, UfoBuffer **inputs, UfoRequisition *requisition,
                                     GError **error)
{
    ufo_ir_shell_method_requisition (SELF (task)->base.projector, inputs, requisition, error);
}

static guint
ufo_ir_asdpocs_task_get_num_inputs (UfoTask *task)
{
    return 1;
}

static guint
ufo_ir_asdpocs_task_get_num_dimensions (UfoTask *task, guint input)
{
    g_return_val_if_fail (input == 0, 0);
    return 2;
}

static UfoTaskMode
ufo_ir_asdpocs_task_get_mode (UfoTask *task)
{
    return UFO_TASK_MODE_PROCESSOR | UFO_TASK_MODE_CPU;
}

static gboolean
ufo_ir_asdpocs_task_process (UfoTask *task, UfoBuffer **inputs, UfoBuffer *output, UfoRequisition *requisition)
{
    UfoIrAsdpocsTask *self = SELF (task);
    ufoir_projector *proj = ufo_ir_shell_projector (self->base.projector, NULL);
    ufoir_asdpocs_params prm;
    size_t dims[2];
    guint sart_iterations = 10;
    gfloat sart_relaxation = 0.25f;

    if (proj == NULL || self->df_minimizer == NULL)
        return ufo_ir_method_shell_done ("asdpocs", UFOIR_ERR_STATE);
    g_object_get (self->df_minimizer, "num-iterations", &sart_iterations, "relaxation_factor", &sart_relaxation,
                  NULL);
    ufoir_asdpocs_params_init (&prm);
    prm.num_iterations = self->base.num_iterations;
    prm.beta = self->beta;
    prm.beta_red = self->beta_red;
    prm.alpha = self->alpha;
    prm.alpha_red = self->alpha_red;
    prm.r_max = self->r_max;
    prm.ng = self->ng;
    prm.positive_constraint = self->positive_constraint ? 1 : 0;
    prm.df_minimizer.num_iterations = sart_iterations;
    prm.df_minimizer.relaxation_factor = sart_relaxation;
    prm.norm_mode = ufo_ir_shell_norm_mode (self->norm_mode);
    ufo_ir_method_shell_dims (inputs[0], dims);
    return ufo_ir_method_shell_done ("asdpocs",
        ufoir_asdpocs_process (proj, &prm, ufo_buffer_get_host_array (inputs[0], NULL), dims,
                               ufo_buffer_get_host_array (output, NULL), 1));
}

static void
ufo_task_interface_init (UfoTaskIface *iface)
{
    iface->setup = ufo_ir_asdpocs_task_setup;
    iface->get_requisition = ufo_ir_asdpocs_task_get_requisition;
    iface->get_num_inputs = ufo_ir_asdpocs_task_get_num_inputs;
    iface->get_num_dimensions = ufo_ir_asdpocs_task_get_num_dimensions;
    iface->get_mode = ufo_ir_asdpocs_task_get_mode;
    iface->process = ufo_ir_asdpocs_task_process;
}

static void
ufo_ir_asdpocs_task_class_init (UfoIrAsdpocsTaskClass *klass)
{
    GObjectClass *oclass = G_OBJECT_CLASS (klass);

    oclass->set_property = ufo_ir_asdpocs_task_set_property;
    oclass->get_property = ufo_ir_asdpocs_task_get_property;
    oclass->dispose = ufo_ir_asdpocs_task_dispose;
    oclass->finalize = ufo_ir_asdpocs_task_finalize;
    ufo_ir_method_shell_install (oclass);
    g_object_class_install_property (oclass, PROP_BETA,
        g_param_spec_float ("beta", "Beta", "Beta", 0.0f, G_MAXFLOAT, 1.0f, G_PARAM_READWRITE));
    g_object_class_install_property (oclass, PROP_BETA_RED,
        g_param_spec_float ("beta_red", "Beta red", "Beta red", 0.0f, G_MAXFLOAT, 0.995f, G_PARAM_READWRITE));
    g_object_class_install_property (oclass, PROP_NG,
        g_param_spec_uint ("ng", "NG", "NG", 0, 1000, 20, G_PARAM_READWRITE));
    g_object_class_install_property (oclass, PROP_ALPHA,
        g_param_spec_float ("alpha", "Alpha", "Alpha", 0.0f, G_MAXFLOAT, 0.2f, G_PARAM_READWRITE));
    g_object_class_install_property (oclass, PROP_ALPHA_RED,
        g_param_spec_float ("alpha_red", "Alpha Red", "Alpha Red", 0.0f, G_MAXFLOAT, 0.95f, G_PARAM_READWRITE));
    g_object_class_install_property (oclass, PROP_R_MAX,
        g_param_spec_float ("r_max", "R-max", "R-max", 0.0f, G_MAXFLOAT, 0.95f, G_PARAM_READWRITE));
    g_object_class_install_property (oclass, PROP_POSITIVE_CONSTRAINT,
        g_param_spec_boolean ("positive_constraint", "Impose positive constraint", "Impose positive constraint",
                              TRUE, G_PARAM_READWRITE));
    g_object_class_install_property (oclass, PROP_DF_MINIMIZER,
        g_param_spec_object ("df_minimizer", "Current minimizer", "Current minimizer", G_TYPE_OBJECT,
                             G_PARAM_READWRITE));
    g_object_class_install_property (oclass, PROP_NORM_MODE,
        g_param_spec_string ("norm-mode", "Norm arithmetic", "fp64 (default) or compat", "fp64",
                             G_PARAM_READWRITE));
}

static void
ufo_ir_asdpocs_task_init (UfoIrAsdpocsTask *self)
{
    ufo_ir_method_shell_init (&self->base);
    self->beta = 1.0f;
    self->beta_red = 0.995f;
    self->alpha = 0.2f;
    self->alpha_red = 0.95f;
    self->r_max = 0.95f;
    self->ng = 20;
    self->positive_constraint = TRUE;
    self->df_minimizer = NULL;
    self->norm_mode = g_strdup ("fp64");
}
