/*
 * Minimal GLib stand-in (GTree subset) so the reference's STL reader
 * (src/geo3d.c:229-401) compiles without GLib.  Test infrastructure only.
 *
 * The reference uses the tree as an ordered map keyed by its own comparison
 * function and numbers vertices/edges by g_tree_nnodes() at insertion time,
 * so any ordered map with the same comparator reproduces its indices.
 */
#ifndef ORACLE_SHIM_GLIB_H
#define ORACLE_SHIM_GLIB_H

#ifdef __cplusplus
extern "C" {
#endif

typedef void *gpointer;
typedef const void *gconstpointer;
typedef int gint;
typedef int gboolean;
typedef gint (*GCompareDataFunc)(gconstpointer a, gconstpointer b, gpointer user_data);
typedef gboolean (*GTraverseFunc)(gpointer key, gpointer value, gpointer data);
typedef void (*GDestroyNotify)(gpointer data);
typedef struct _GTree GTree;

#define G_GNUC_UNUSED __attribute__((unused))

void g_free(gpointer mem);
GTree *g_tree_new_full(GCompareDataFunc key_compare, gpointer key_compare_data,
                       GDestroyNotify key_destroy, GDestroyNotify value_destroy);
gpointer g_tree_lookup(GTree *tree, gconstpointer key);
void g_tree_insert(GTree *tree, gpointer key, gpointer value);
gint g_tree_nnodes(GTree *tree);
void g_tree_foreach(GTree *tree, GTraverseFunc func, gpointer user_data);
void g_tree_destroy(GTree *tree);

#ifdef __cplusplus
}
#endif

#endif
