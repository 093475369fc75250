/*
 * Binary structure-of-arrays snapshot of one explicit-MPM state ("MPMSNAP1").
 *
 * Test infrastructure for the oracle: the headless reference driver
 * (oracle/ref_driver.cpp) and the CPU restatement (oracle/mpm_oracle.c) both
 * read and write this layout, so a state at step k can be handed between the
 * reference, the restatement and the CUDA engine without loss.  The product's
 * own reader/writer of the same layout is code_mpm_gb300/snapshot.py.
 *
 * The field set is the state of the reference's data model:
 *   particles  MaterialPoint_BC.h:25-85 (position, velocity, external force,
 *              mass, volume, deformation gradient, Voigt stress/strain/plastic
 *              strain, energies, isotropic back-stress, contact mass gradient,
 *              strain rate, displacement-control flags and multiplier)
 *   nodes      GridPoint.h:6-45 (fixed flags, friction, mass, momentum,
 *              velocity, force, reaction force, mass gradient, active and
 *              contact flags)
 *   materials  Material_BC.h:13-35
 *   timeline   TimeLine.h:33-46
 *
 * Layout (little-endian): a fixed header, then every array back to back in
 * the order of the MPMSNAP_FIELDS table below.  Per-particle vectors are
 * stored n x k row-major (the k components of particle 0 first).  The 3x3
 * deformation gradient is stored in glm's column-major element order
 * (F[c][r] at offset 3*c + r).  With MPMSNAP_HAS_FE in the header flags, the
 * elastic deformation gradient (MaterialPoint_BC.h:65, the state of the
 * large-strain pass 2) follows as one more [n][9] array; without it, it is
 * the identity.
 */
#ifndef MPM_SNAPSHOT_H
#define MPM_SNAPSHOT_H

#include <stddef.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#define MPMSNAP_MAGIC "MPMSNAP1"
#define MPMSNAP_HAS_FE 1u /* header flags: the elastic deformation gradient block follows */

/* particle flag bits */
#define MPM_PF_DC_X 1u     /* b3_DisplacementControl.x */
#define MPM_PF_DC_Y 2u     /* b3_DisplacementControl.y */
#define MPM_PF_DC_Z 4u     /* b3_DisplacementControl.z */
#define MPM_PF_DC_SKIP 8u  /* b_DisplacementControl (contact path skips G2P) */
#define MPM_PF_SURFACE 16u /* b_Surface */

/* node flag bits (fixed) */
#define MPM_NF_FIX_X 1u
#define MPM_NF_FIX_Y 2u
#define MPM_NF_FIX_Z 4u
/* node state bits */
#define MPM_NS_ACTIVE 1u
#define MPM_NS_CONTACT 2u
#define MPM_NS_POSITIVE 4u
#define MPM_NS_NEGATIVE 8u

typedef struct mpmsnap_material {
    int32_t type; /* 0 elastic, 3 perfectly plastic, 4 von Mises hardening */
    int32_t pad;
    double density, E, nu, yield, C0, C1;
} mpmsnap_material;

typedef struct mpmsnap_header {
    char magic[8];
    uint32_t version;
    uint32_t contact; /* which solver the state was last advanced by (info) */
    double length[3];
    int32_t cells[3];
    int32_t pad0;
    double time, dt_max, mass_min, damping;
    int64_t step;
    uint64_t n_particles;
    uint64_t n_nodes;
    uint32_t n_materials;
    uint32_t n_timeline;
    uint32_t n_dc;
    uint32_t flags; /* MPMSNAP_HAS_FE */
} mpmsnap_header;

typedef struct mpmsnap {
    mpmsnap_header h;
    mpmsnap_material* materials; /* [n_materials] */
    double* tl_time;             /* [n_timeline] */
    double* tl_vel;              /* [n_timeline][3] */
    /* particles */
    double *pos, *vel, *fext;       /* [n][3] */
    double *mass, *vol, *vol0;      /* [n] */
    double* F;                      /* [n][9] */
    double *stress, *strain, *eps_p; /* [n][6] */
    double *e_strain, *e_strain_max, *e_strain_ti, *e_plastic, *backstress; /* [n] */
    double* mp_mass_gradient;       /* [n][3] */
    double* strain_rate;            /* [n][6] */
    int32_t* material;              /* [n] */
    uint8_t* pflags;                /* [n] */
    float* dc_mult;                 /* [n] */
    uint32_t* dc_list;              /* [n_dc] */
    /* nodes */
    uint8_t* fixed;     /* [nn] */
    double* friction;   /* [nn] */
    double* g_mass;     /* [nn] */
    double *g_mom, *g_vel, *g_force, *g_force_temp, *g_mass_gradient; /* [nn][3] */
    uint8_t* g_state;   /* [nn] */
    double* F_elastic;  /* [n][9], identity unless the file holds it (not in MPMSNAP_FIELDS) */
} mpmsnap;

/* (pointer member offset, element size, components, count selector: 0 particles, 1 nodes, 2 materials, 3 timeline, 4 dc) */
typedef struct mpmsnap_field {
    size_t off;
    size_t esize;
    size_t comp;
    int count;
} mpmsnap_field;

#define MPMSNAP_F(member, esz, comp, cnt) {offsetof(mpmsnap, member), esz, comp, cnt}
static const mpmsnap_field MPMSNAP_FIELDS[] = {
    MPMSNAP_F(materials, sizeof(mpmsnap_material), 1, 2),
    MPMSNAP_F(tl_time, 8, 1, 3),
    MPMSNAP_F(tl_vel, 8, 3, 3),
    MPMSNAP_F(pos, 8, 3, 0),
    MPMSNAP_F(vel, 8, 3, 0),
    MPMSNAP_F(fext, 8, 3, 0),
    MPMSNAP_F(mass, 8, 1, 0),
    MPMSNAP_F(vol, 8, 1, 0),
    MPMSNAP_F(vol0, 8, 1, 0),
    MPMSNAP_F(F, 8, 9, 0),
    MPMSNAP_F(stress, 8, 6, 0),
    MPMSNAP_F(strain, 8, 6, 0),
    MPMSNAP_F(eps_p, 8, 6, 0),
    MPMSNAP_F(e_strain, 8, 1, 0),
    MPMSNAP_F(e_strain_max, 8, 1, 0),
    MPMSNAP_F(e_strain_ti, 8, 1, 0),
    MPMSNAP_F(e_plastic, 8, 1, 0),
    MPMSNAP_F(backstress, 8, 1, 0),
    MPMSNAP_F(mp_mass_gradient, 8, 3, 0),
    MPMSNAP_F(strain_rate, 8, 6, 0),
    MPMSNAP_F(material, 4, 1, 0),
    MPMSNAP_F(pflags, 1, 1, 0),
    MPMSNAP_F(dc_mult, 4, 1, 0),
    MPMSNAP_F(dc_list, 4, 1, 4),
    MPMSNAP_F(fixed, 1, 1, 1),
    MPMSNAP_F(friction, 8, 1, 1),
    MPMSNAP_F(g_mass, 8, 1, 1),
    MPMSNAP_F(g_mom, 8, 3, 1),
    MPMSNAP_F(g_vel, 8, 3, 1),
    MPMSNAP_F(g_force, 8, 3, 1),
    MPMSNAP_F(g_force_temp, 8, 3, 1),
    MPMSNAP_F(g_mass_gradient, 8, 3, 1),
    MPMSNAP_F(g_state, 1, 1, 1),
};
#define MPMSNAP_NFIELDS (sizeof(MPMSNAP_FIELDS) / sizeof(MPMSNAP_FIELDS[0]))

static size_t mpmsnap_count(const mpmsnap_header* h, int sel) {
    switch (sel) {
        case 0: return (size_t)h->n_particles;
        case 1: return (size_t)h->n_nodes;
        case 2: return (size_t)h->n_materials;
        case 3: return (size_t)h->n_timeline;
        default: return (size_t)h->n_dc;
    }
}

static void** mpmsnap_slot(mpmsnap* s, size_t i) { return (void**)((char*)s + MPMSNAP_FIELDS[i].off); }

/* Allocate every array (zero-filled) for the counts already in s->h. */
static int mpmsnap_alloc(mpmsnap* s) {
    for (size_t i = 0; i < MPMSNAP_NFIELDS; ++i) {
        size_t bytes = mpmsnap_count(&s->h, MPMSNAP_FIELDS[i].count) * MPMSNAP_FIELDS[i].esize * MPMSNAP_FIELDS[i].comp;
        void* p = calloc(bytes ? bytes : 1, 1);
        if (!p) return -1;
        *mpmsnap_slot(s, i) = p;
    }
    const size_t n = (size_t)s->h.n_particles;
    s->F_elastic = (double*)calloc(n ? n * 9 : 1, sizeof(double));
    if (!s->F_elastic) return -1;
    for (size_t p = 0; p < n; ++p) s->F_elastic[9 * p] = s->F_elastic[9 * p + 4] = s->F_elastic[9 * p + 8] = 1.0;
    return 0;
}

static void mpmsnap_free(mpmsnap* s) {
    for (size_t i = 0; i < MPMSNAP_NFIELDS; ++i) {
        free(*mpmsnap_slot(s, i));
        *mpmsnap_slot(s, i) = NULL;
    }
    free(s->F_elastic);
    s->F_elastic = NULL;
}

static int mpmsnap_read(const char* path, mpmsnap* s) {
    FILE* f = fopen(path, "rb");
    if (!f) return -1;
    memset(s, 0, sizeof(*s));
    if (fread(&s->h, sizeof(s->h), 1, f) != 1 || memcmp(s->h.magic, MPMSNAP_MAGIC, 8) != 0 || s->h.version != 1) {
        fclose(f);
        return -2;
    }
    if (mpmsnap_alloc(s) != 0) {
        fclose(f);
        return -3;
    }
    for (size_t i = 0; i < MPMSNAP_NFIELDS; ++i) {
        size_t nel = mpmsnap_count(&s->h, MPMSNAP_FIELDS[i].count) * MPMSNAP_FIELDS[i].comp;
        if (nel && fread(*mpmsnap_slot(s, i), MPMSNAP_FIELDS[i].esize, nel, f) != nel) {
            fclose(f);
            return -4;
        }
    }
    const size_t nfe = (size_t)s->h.n_particles * 9;
    if ((s->h.flags & MPMSNAP_HAS_FE) && nfe && fread(s->F_elastic, 8, nfe, f) != nfe) {
        fclose(f);
        return -4;
    }
    fclose(f);
    return 0;
}

static int mpmsnap_write(const char* path, const mpmsnap* s) {
    FILE* f = fopen(path, "wb");
    if (!f) return -1;
    if (fwrite(&s->h, sizeof(s->h), 1, f) != 1) {
        fclose(f);
        return -2;
    }
    for (size_t i = 0; i < MPMSNAP_NFIELDS; ++i) {
        size_t nel = mpmsnap_count(&s->h, MPMSNAP_FIELDS[i].count) * MPMSNAP_FIELDS[i].comp;
        void* p = *(void* const*)((const char*)s + MPMSNAP_FIELDS[i].off);
        if (nel && fwrite(p, MPMSNAP_FIELDS[i].esize, nel, f) != nel) {
            fclose(f);
            return -3;
        }
    }
    const size_t nfe = (size_t)s->h.n_particles * 9;
    if ((s->h.flags & MPMSNAP_HAS_FE) && nfe && fwrite(s->F_elastic, 8, nfe, f) != nfe) {
        fclose(f);
        return -3;
    }
    fclose(f);
    return 0;
}

#endif /* MPM_SNAPSHOT_H */
