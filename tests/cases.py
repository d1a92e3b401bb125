"""Small model instances shared by the tests (sizes the oracle finishes in seconds)."""
from kapdqmc_gb300 import tU_Hubbard_Para, tUV_Hubbard_Para, tV_Hubbard_Para


def tu_square(Nt_half=1.0, BS=5, U=4.0, site=(2, 4), flux=0.0):
    return tU_Hubbard_Para(Ht=1.0, Hu1=U, Hu2=U, Δt=0.1, Θrelax=Nt_half, Θquench=0.0,
                           Lattice="SQUARE45", site=list(site), BatchSize=BS, Initial="H0", flux=flux)


def tu_honeycomb(BS=5):
    return tU_Hubbard_Para(Ht=1.0, Hu1=4.0, Hu2=4.0, Δt=0.1, Θrelax=1.0, Θquench=0.0,
                           Lattice="HoneyComb120", site=[3, 3], BatchSize=BS, Initial="H0")


def tu_quench():
    # the reference's test parameters: src test/tU/HCtU_runtests.jl:12-13
    return tU_Hubbard_Para(Ht=1.0, Hu1=0.0, Hu2=3.8, Θrelax=0.4, Θquench=0.4, Lattice="HoneyComb120",
                           site=[3, 3], Δt=0.1, BatchSize=10, Initial="H0")


def tv_honeycomb(BS=5, V=1.0):
    return tV_Hubbard_Para(Ht=1.0, Hv1=V, Hv2=V, Δt=0.1, Θrelax=1.0, Θquench=0.0,
                           Lattice="HoneyComb120", site=[3, 3], BatchSize=BS, Initial="H0")


def tuv_honeycomb(U=4.0, V=0.5):
    return tUV_Hubbard_Para(Ht=1.0, Hu=U, Hv=V, Lattice="HoneyComb120", site=[3, 3], Δt=0.1, Θ=1.0,
                            BatchSize=5, Initial="H0")


def tuv_square():
    return tUV_Hubbard_Para(Ht=1.0, Hu=4.0, Hv=0.5, Lattice="SQUARE45", site=[2, 4], Δt=0.1, Θ=1.0,
                            BatchSize=5, Initial="H0", allow_marginal=True)


def c1():
    """t-U 4x4 square, U=4, dt=0.1, 2Θ=10 (100 slices), n_wrap=10."""
    return tU_Hubbard_Para(Ht=1.0, Hu1=4.0, Hu2=4.0, Δt=0.1, Θrelax=5.0, Θquench=0.0,
                           Lattice="SQUARE45", site=[2, 4], BatchSize=10, Initial="H0")


def c2():
    """t-V 6x6 honeycomb, V=1, dt=0.05, 2Θ=20 (400 slices), n_wrap=10."""
    return tV_Hubbard_Para(Ht=1.0, Hv1=1.0, Hv2=1.0, Δt=0.05, Θrelax=10.0, Θquench=0.0,
                           Lattice="HoneyComb120", site=[6, 6], BatchSize=10, Initial="H0")


def c3():
    """t-U 12x12 square, U=8, dt=0.05, 2Θ=16 (320 slices), n_wrap=8."""
    return tU_Hubbard_Para(Ht=1.0, Hu1=8.0, Hu2=8.0, Δt=0.05, Θrelax=8.0, Θquench=0.0,
                           Lattice="SQUARE45", site=[6, 12], BatchSize=8, Initial="H0")


def c4():
    """t-UV 8x8 square, U=4, V=0.5, dt=0.1, 2Θ=20 (200 slices), marginal stability."""
    return tUV_Hubbard_Para(Ht=1.0, Hu=4.0, Hv=0.5, Lattice="SQUARE45", site=[4, 8], Δt=0.1, Θ=10.0,
                            BatchSize=10, Initial="H0", allow_marginal=True)


def c5():
    """t-U 9x9 honeycomb, U=4, dt=0.1, 2Θ=20 (200 slices), n_wrap=10."""
    return tU_Hubbard_Para(Ht=1.0, Hu1=4.0, Hu2=4.0, Δt=0.1, Θrelax=10.0, Θquench=0.0,
                           Lattice="HoneyComb120", site=[9, 9], BatchSize=10, Initial="H0")


def tu_square90_flux():
    # the reference's π-flux test lattice (test/tU/□tU_runtests.jl:44-45), 4x4 instead of 6x6
    return tU_Hubbard_Para(Ht=1.0, Hu1=4.0, Hu2=4.0, Θrelax=1.0, Θquench=0.0, Lattice="SQUARE90",
                           site=[4, 4], Δt=0.1, BatchSize=5, Initial="H0", flux=3.141592653589793)


def tu_honeycomb60():
    return tU_Hubbard_Para(Ht=1.0, Hu1=4.0, Hu2=4.0, Δt=0.1, Θrelax=1.0, Θquench=0.0,
                           Lattice="HoneyComb60", site=[3, 3], BatchSize=5, Initial="H0")


def tv_honeycomb60():
    return tV_Hubbard_Para(Ht=1.0, Hv1=1.0, Hv2=1.0, Δt=0.1, Θrelax=1.0, Θquench=0.0,
                           Lattice="HoneyComb60", site=[3, 3], BatchSize=5, Initial="H0")


def tuv_honeycomb60():
    return tUV_Hubbard_Para(Ht=1.0, Hu=4.0, Hv=0.5, Lattice="HoneyComb60", site=[3, 3], Δt=0.1, Θ=1.0,
                            BatchSize=5, Initial="H0")


# Lattices small enough for the exact Fock-space sum (Ns <= 12)
def tu_hc8(U=4.0):
    return tU_Hubbard_Para(Ht=1.0, Hu1=U, Hu2=U, Δt=0.1, Θrelax=1.0, Θquench=0.0,
                           Lattice="HoneyComb120", site=[2, 2], BatchSize=5, Initial="H0")


def tu_hc8_quench():
    return tU_Hubbard_Para(Ht=1.0, Hu1=0.0, Hu2=3.8, Θrelax=0.4, Θquench=0.4, Lattice="HoneyComb120",
                           site=[2, 2], Δt=0.1, BatchSize=4, Initial="H0")


def tu_sq8():
    return tU_Hubbard_Para(Ht=1.0, Hu1=4.0, Hu2=4.0, Θrelax=1.0, Θquench=0.0, Lattice="SQUARE45",
                           site=[2, 2], Δt=0.1, BatchSize=5, Initial="H0")


def tu_sq8_flux():
    return tU_Hubbard_Para(Ht=1.0, Hu1=4.0, Hu2=4.0, Θrelax=1.0, Θquench=0.0, Lattice="SQUARE90",
                           site=[2, 2], Δt=0.1, BatchSize=5, Initial="H0", flux=3.141592653589793)


def tu_hc12():
    return tU_Hubbard_Para(Ht=1.0, Hu1=4.0, Hu2=4.0, Θrelax=1.0, Θquench=0.0, Lattice="HoneyComb120",
                           site=[2, 3], Δt=0.1, BatchSize=5, Initial="H0")


def tv_hc8(V=1.0):
    return tV_Hubbard_Para(Ht=1.0, Hv1=V, Hv2=V, Δt=0.1, Θrelax=1.0, Θquench=0.0,
                           Lattice="HoneyComb120", site=[2, 2], BatchSize=5, Initial="H0")


def tuv_hc8():
    return tUV_Hubbard_Para(Ht=1.0, Hu=4.0, Hv=0.5, Lattice="HoneyComb120", site=[2, 2], Δt=0.1, Θ=1.0,
                            BatchSize=5, Initial="H0")


def tuv_hc8_real():
    # U < 0: the real t-UV sweep (det^2 weights with the exp(-(a+1) eta) field factor)
    return tUV_Hubbard_Para(Ht=1.0, Hu=-4.0, Hv=0.3, Lattice="HoneyComb120", site=[2, 2], Δt=0.1, Θ=1.0,
                            BatchSize=5, Initial="H0")
