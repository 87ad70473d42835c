"""Scene texts, valid and malformed, whose load_scene outcome pins the host
parser's messages to the reference's (gen_golden.py, group `messages`, runs
the reference's load_scene on each; tests/test_host_layer.py compares)."""

# Lines every case may use: a texture and a volume material.
PRELUDE = "texture t solid 0.5 0.5 0.5\nmaterial haze volume 0.9 0.9 0.9\n"

CASES = [
    # valid
    "sphere 0 0 0 1 scale 2 translate 1 1 1 rotate_y 30",
    "aspect_ratio 16/9\nsphere 0 0 0 1",
    "material m principled color 0.5 0.5 0.5 metallic texture t roughness 0.3 clearcoat 1 "
    "clearcoat_color 0.5 0.5 0.5\nsphere 0 0 0 1 m",
    "material m lambertian 1 1 1 normal_map t\nsphere 0 0 0 1 m",
    "material m metal Au 0.3\nbox 0 0 0 1 1 1 m rotate 20 1 1 0",
    "camera lookfrom 1 2 3 lookat 0 0 0 vup 0 1 0 vfov 30 aperture 1 focus 4 blades 6 blade_rotation 10\n"
    "sphere 0 0 0 1",
    "sun elevation 30 azimuth 20 intensity 2 color 1 0.9 0.8 angle 2 disk off\nsky atmosphere rayleigh 2\n"
    "ground height -1\nsphere 0 0 0 1",
    "bounces diffuse 2 specular 3 scatter 4\nsphere 0 0 0 1",
    "medium 0.1 sphere 0 0 0 1 haze scale 1 2 1\nfog 0.01 haze\nsphere 0 0 0 1",
    # malformed
    "image_width 0", "image_width abc", "image_width 10 20", "aspect_ratio", "aspect_ratio 16/x",
    "aspect_ratio -1", "samples_per_pixel 0", "max_depth -3",
    "camera lookfrom 1 2", "camera vfov 200", "camera frobnicate 3", "camera blades 2",
    "vfov 0", "aperture -1", "focus 0", "background 1 1", "light_selection random",
    "environment", "environment sky.hdr brightness 2", "environment missing.hdr",
    "sun elevation 100", "sun disk maybe", "sun wobble 3", "sun elevation 45 azimuth 30 off color 1 1",
    "sky", "sky uniform 1 1", "sky atmosphere mie_g 1.5", "sky plasma",
    "ground height", "ground nosuch", "ground off height x", "style fancy",
    "bounces diffuse -1", "bounces bright 2", "transparent_shadows maybe",
    "height_fog 0 8 haze", "height_fog 0.1 8 haze ceiling 3",
    "material m lambertian 1 1 1\nheight_fog 0.1 8 m",
    "bloom -1", "bloom 0.3 radius 0", "vignette -0.1", "exposure high", "tonemap filmic", "normal_maps maybe",
    "texture u", "texture u solid 1 1", "texture u checker 0 1 1 1 0 0 0", "texture u image",
    "texture u image x.png srgb", "texture u image missing.png", "texture u wood",
    "material m", "material m plastic", "material m lambertian 1 1", "material m lambertian texture nosuch",
    "material m lambertian texture", "material m lambertian 1 1 1 normal_map",
    "material m lambertian 1 1 1 bump t", "material m lambertian 1 1 1 normal_map t junk",
    "material m metal 1 1 1", "material m metal Zn 0.3", "material m metal Al -1",
    "material m dielectric 0", "material m dielectric 1.5 color 0 1 1", "material m dielectric 1.5 shiny 2",
    "material m dielectric 1.5 roughness", "material m thin_glass 1.5 color 2 1 1",
    "material m thin_glass 1.5 tint 1 1 1",
    "material m principled metallic 2", "material m principled sparkle 1",
    "material m principled conductor Zn", "material m principled clearcoat_roughness 0.1",
    "material m principled texture nosuch", "material m principled texture",
    "material m volume 1 1", "material m volume 1 1 1 g 1", "material m emissive 1 1 1 spread 0",
    "material m emissive 1 1",
    "sphere 0 0 0", "sphere 0 0 0 0", "sphere 0 0 0 1 nope", "sphere 0 0 0 1 translate 1 2",
    "sphere 0 0 0 1 scale 0", "sphere 0 0 0 1 scale 1 2", "sphere 0 0 0 1 rotate 30 0 0 0",
    "sphere 0 0 0 1 wiggle 3", "sphere 0 0 0 1 haze translate 1 2 3 scale",
    "quad 0 0 0 1 0 0 2 0 0", "quad 0 0 0 1 0 0", "box 0 0 0 1 1",
    "medium 0 sphere 0 0 0 1 haze", "medium 0.1 cone 0 0 0 1", "medium 0.1 sphere 0 0 0 0 haze",
    "medium 0.1 box 0 0 0 1 1", "material m lambertian 1 1 1\nmedium 0.1 box 0 0 0 1 1 1 m",
    "fog 0 haze", "fog 0.1 nosuch",
    "mesh", "mesh missing.obj", "mesh x.obj replace a", "material m lambertian 1 1 1\nmesh x.obj replace a m",
    "vox", "vox missing.vox", "frobnicate 3", "image_width 10",
    "material l emissive 1 1 1\nsphere 0 0 0 1 l scale 1 2 1",
    "sphere 0 0 0 1\ncamera lookfrom 0 0 0 lookat 0 0 0",
]
