# Runs the reference (Stencils.jl) on the committed seeded inputs and compares its results with the
# committed oracle outputs, case by case.  For a host with Julia and the reference's environment
# (Stencils, StaticArrays, Statistics, BFloat16s); neither the build container nor the GPU hosts have
# Julia, so this script has not been run.  Bit-exact cases compare bit patterns; "kdot-f32" cases report
# the largest difference relative to the magnitude of the result.
#
#     julia --project=<environment with Stencils> tests/golden/seeded/run_reference.jl
using TOML, Stencils, StaticArrays, Statistics, BFloat16s

const DIR = @__DIR__
const M = TOML.parsefile(joinpath(DIR, "manifest.toml"))
const ELTYPES = Dict("Float64" => Float64, "Float32" => Float32, "UInt8" => UInt8, "BFloat16" => BFloat16)

function load(case, key)
    e = M[case]["arrays"][key]
    T = ELTYPES[e["eltype"]]
    v = reinterpret(T, read(joinpath(DIR, e["file"])))
    return copy(reshape(v, Tuple(e["shape"])))
end

life(h) = (s = sum(neighbors(h)); UInt8(s == 3 || (center(h) == 1 && s == 2)))
diffuse(h) = center(h) + 0.1f0 * (sum(neighbors(h)) - 6 * center(h))
gauss(a) = Kernel(Window(3), SVector{49}(load(a, "weights")))
layered() = Layered(x=Layered(a=Moore(1), b=Window(2)), y=Circle(3))

const RUN = Dict(
    "mean_blur_f64" => c -> mapstencil(mean, StencilArray(load(c, "A"), Window(1);
                                                         boundary=Remove(0.0), padding=Conditional())),
    "life_u8" => c -> begin
        S = SwitchingStencilArray(load(c, "A"), Moore(1); boundary=Wrap(), padding=Halo{:out}())
        for _ in 1:10
            S = mapstencil!(life, S)
        end
        parent(S)[2:end-1, 2:end-1]
    end,
    "gauss7_f32" => c -> mapstencil(kernelproduct, StencilArray(load(c, "A"), gauss(c); boundary=Remove(0f0))),
    "gauss7_bf16" => c -> BFloat16.(mapstencil(kernelproduct,
                                               StencilArray(load(c, "A"), gauss(c); boundary=Remove(BFloat16(0))))),
    "diffusion3d_f32" => c -> begin
        S = SwitchingStencilArray(load(c, "A"), VonNeumann(1, 3); boundary=Wrap())
        for _ in 1:5
            S = mapstencil!(diffuse, S)
        end
        parent(S)
    end,
    "circle3_reflect_f32" => c -> mapstencil(mean, StencilArray(load(c, "A"), Circle(3);
                                                               boundary=Reflect(), padding=Halo{:out}())),
    "two_array_f64" => c -> mapstencil((a, b) -> center(a) + 0.1 * sum(b),
                                       StencilArray(load(c, "A"), Moore(1); boundary=Remove(0.0)),
                                       StencilArray(load(c, "B"), Moore(1); boundary=Remove(0.0))),
    "scatter_center_f64" => c -> scatterstencil!(h -> map(_ -> center(h), neighbors(h)), +, load(c, "dest0"),
                                                 StencilArray(load(c, "A"), Moore(1); boundary=Wrap())),
    "layered_f64" => c -> mapstencil(l -> mean(l.x.a) + 0.5 * sum(l.y),
                                     StencilArray(load(c, "A"), layered(); boundary=Wrap())),
)

bits(x::AbstractArray{T}) where T = reinterpret(sizeof(T) == 8 ? UInt64 : sizeof(T) == 4 ? UInt32 :
                                                sizeof(T) == 2 ? UInt16 : UInt8, vec(x))

failures = 0
for case in sort(collect(keys(M)))
    want = load(case, "out")
    got = RUN[case](case)
    if M[case]["tolerance"] == "bit-exact"
        ok = size(got) == size(want) && bits(collect(got)) == bits(want)
        println(rpad(case, 24), ok ? "bit-exact" : "DIFFERS")
        global failures += !ok
    else
        g, w = Float64.(collect(got)), Float64.(want)
        rel = maximum(abs.(g .- w)) / max(maximum(abs.(w)), eps())
        println(rpad(case, 24), "max |diff| / max |out| = ", rel)
    end
end
exit(failures == 0 ? 0 : 1)
